// umma.cuh -- inline-PTX helpers for the 5th-generation tensor cores (tcgen05) of
// sm_100-family GPUs, written from the public PTX ISA: shared-memory matrix
// descriptors, the instruction descriptor of kind::f16, tensor-memory (TMEM)
// allocation, MMA issue and commit, TMEM loads, mbarriers with bounded waits, and the
// proxy / thread-sync fences these need.
//
// Operand layout used throughout ("no swizzle", K-major): a matrix of R rows x 16
// bf16 columns (K) is a grid of core matrices of 8 rows x 16 bytes (8 bf16 of K),
// each stored as 128 contiguous bytes (row r at +16 r).  Core matrix (i, j) -- rows
// 8i..8i+7, K columns 8j..8j+7 -- starts at start + i * SBO + j * LBO.
#pragma once

#include <cstdint>

namespace dxmcg {
namespace umma {

    __device__ __forceinline__ uint32_t smemAddr(const void* p)
    {
        return static_cast<uint32_t>(__cvta_generic_to_shared(p));
    }

    // Shared-memory matrix descriptor: start address, leading byte offset (between
    // core matrices along K), stride byte offset (between core matrices along M or
    // N), descriptor version 1, no swizzle.  All three are in 16-byte units.
    __device__ __forceinline__ uint64_t smemDescriptor(uint32_t saddr, uint32_t lbo, uint32_t sbo)
    {
        uint64_t d = 0;
        d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
        d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
        d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
        d |= 1ull << 46; // version
        return d;       // base offset 0, LBO mode 0, layout type 0 (no swizzle)
    }

    // Instruction descriptor of kind::f16: D in FP32, A and B bf16, both K-major,
    // M x N (M = 64 or 128; N a multiple of 8 for M = 64, of 16 for M = 128).
    __host__ __device__ constexpr uint32_t instrDescriptorBf16(int M, int N)
    {
        return (1u << 4)                                  // D format: F32
            | (1u << 7)                                   // A format: BF16
            | (1u << 10)                                  // B format: BF16
            | (static_cast<uint32_t>(N >> 3) << 17)      // N / 8
            | (static_cast<uint32_t>(M >> 4) << 24);     // M / 16
    }

    // ---- tensor memory (one warp allocates and frees; ncols a power of 2 >= 32)
    __device__ __forceinline__ void tmemAlloc(uint32_t* dstSmem, uint32_t ncols)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(dstSmem)),
            "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    __device__ __forceinline__ void tmemFree(uint32_t taddr, uint32_t ncols)
    {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols));
    }

    __device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
    __device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
    // generic-proxy writes to shared memory made visible to the tensor core (async proxy)
    __device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

    // ---- MMA: D[tmem] (+)= A[smem] x B[smem]^T, issued by one thread.  Measured on
    // GB300 (152 CTAs, one issuing thread each, constant operands): an M = 128, K = 16
    // MMA takes ~45 SM cycles whatever N up to 64, whatever the number of independent
    // accumulators, the operand layout (no swizzle or 32-byte swizzle) or the A
    // collector; from N = 128 it runs at the full 4096 MAC per cycle (N / 2 cycles).
    // Work shaped as many small-N MMAs should therefore be restacked into larger N.
    enum class Collector { kNone, kFill, kUse, kLastUse };

    template <Collector C>
    __device__ __forceinline__ void mmaBf16(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc,
        bool accumulate)
    {
        const uint32_t acc = accumulate ? 1u : 0u;
        if (C == Collector::kNone)
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                         "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dTmem),
                "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(acc));
        else if (C == Collector::kFill)
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                         "tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%0], %1, %2, %3, p;\n}\n" ::"r"(dTmem),
                "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(acc));
        else if (C == Collector::kUse)
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                         "tcgen05.mma.cta_group::1.kind::f16.collector::a::use [%0], %1, %2, %3, p;\n}\n" ::"r"(dTmem),
                "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(acc));
        else
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                         "tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [%0], %1, %2, %3, p;\n}\n" ::"r"(dTmem),
                "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(acc));
    }

    // the mbarrier at `bar` completes one phase when every MMA this thread issued so far is done
    __device__ __forceinline__ void commit(uint64_t* bar)
    {
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                         smemAddr(bar))
                     : "memory");
    }

    // ---- mbarrier
    __device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smemAddr(bar)), "r"(count) : "memory");
    }
    __device__ __forceinline__ void mbarInval(uint64_t* bar)
    {
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(smemAddr(bar)) : "memory");
    }
    // Waits for the phase with the given parity to complete; gives up after `limit`
    // polls and returns false.
    __device__ __forceinline__ bool mbarWait(uint64_t* bar, uint32_t parity, uint32_t limit)
    {
        const uint32_t a = smemAddr(bar);
        for (uint32_t i = 0; i < limit; ++i) {
            uint32_t done;
            asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                         "selp.u32 %0, 1, 0, p;\n}\n"
                         : "=r"(done)
                         : "r"(a), "r"(parity)
                         : "memory");
            if (done)
                return true;
        }
        return false;
    }

    // Like mbarWait, but also gives up as soon as *abort is set (checked every 64 polls):
    // lets the roles of a warp-specialised CTA leave together when one of them timed out.
    // The first poll is a non-blocking test (mbarrier.test_wait), the later ones may
    // suspend the thread for a while (try_wait): a limit of 1 gives up at once unless
    // the phase has already completed.
    __device__ __forceinline__ bool mbarWaitOrAbort(uint64_t* bar, uint32_t parity, uint32_t limit,
        const volatile int* abort)
    {
        const uint32_t a = smemAddr(bar);
        if (limit == 0u)
            return false;
        uint32_t done;
        asm volatile("{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     "selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done)
            return true;
        for (uint32_t i = 1; i < limit; ++i) {
            asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                         "selp.u32 %0, 1, 0, p;\n}\n"
                         : "=r"(done)
                         : "r"(a), "r"(parity)
                         : "memory");
            if (done)
                return true;
            if ((i & 63u) == 63u && *abort)
                return false;
        }
        return false;
    }
    // one arrival (release semantics: this thread's earlier shared-memory writes are
    // visible to a thread whose wait on the phase succeeds)
    __device__ __forceinline__ void mbarArrive(uint64_t* bar)
    {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smemAddr(bar)) : "memory");
    }

    // ---- TMA: one tiled box of a 5-D tensor map into shared memory, completing on an
    // mbarrier (the caller arms it with the byte count first)
    __device__ __forceinline__ void mbarArriveExpectTx(uint64_t* bar, uint32_t bytes)
    {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smemAddr(bar)), "r"(bytes)
                     : "memory");
    }
    __device__ __forceinline__ void tmaLoad5d(uint32_t dstSmem, const void* tmap, int c0, int c1, int c2, int c3,
        int c4, uint64_t* bar)
    {
        asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                     "%4, %5, %6}], [%7];\n" ::"r"(dstSmem),
            "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smemAddr(bar))
                     : "memory");
    }

    // ---- TMEM -> registers: this warp's 32 lanes (lane base 32 x (warp % 4)), 16 / 32
    // consecutive FP32 columns per thread
    __device__ __forceinline__ void tmemLoad16(uint32_t taddr, float (&v)[16])
    {
        uint32_t r[16];
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                     "[%16];\n"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                     "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                     "=r"(r[14]), "=r"(r[15])
                     : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
        for (int i = 0; i < 16; ++i)
            v[i] = __uint_as_float(r[i]);
    }

    // registers -> TMEM: zeroes 16 consecutive FP32 columns of this warp's 32 lanes
    // (completion is awaited with storeWait before the columns are handed to MMAs)
    __device__ __forceinline__ void tmemZero16(uint32_t taddr)
    {
        const uint32_t z = 0;
        asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};\n" ::"r"(
                         taddr),
            "r"(z)
                     : "memory");
    }
    __device__ __forceinline__ void storeWait() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }

} // namespace umma
} // namespace dxmcg
