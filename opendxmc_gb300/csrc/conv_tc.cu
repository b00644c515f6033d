// conv_tc.cu -- tcgen05 (5th-generation tensor core) kernels of the dose denoiser.
// This part has no counterpart in the reference.
//
// conv3TcKernel is the 3x3x3 convolution (forward, and the input gradient with
// transposed, flipped weights) of channels-last bf16 tensors as an implicit GEMM on
// the tensor cores.  A CTA computes an output brick of 8 (x) x 16 (y) x ZT (z)
// voxels and NT output channels.  Per 16-channel input slice it stages
//   * the zero-padded input halo of 10 x 18 x (ZT + 2) voxels as two planes, one per
//     8-channel half: voxel (hz, hy, hx) of half h at h * plane + ((hz*18 + hy)*10 + hx)*16,
//   * the slice's weights of all 27 taps, the three z-taps of each in-plane tap
//     q = 3 (dy + 1) + (dx + 1) stacked along N: row n = (1 - dz) * NT + co of the
//     B operand of q, half h, at q * 3*NT*32 + h * 3*NT*16 + n * 16,
// in the tensor cores' no-swizzle K-major layout, so that the A operand of a tap is
// the halo seen through a descriptor: row r = 8 y + x of halo plane hz reads halo
// voxel (hz, y + dy + 1, x + dx + 1): 8 consecutive x are one core matrix,
// consecutive y are 160 bytes apart (SBO), the channel halves one plane apart (LBO).
// Output slice o accumulates in TMEM columns [o NT, o NT + NT).  One M = 128 MMA per
// (halo plane hz, in-plane tap q) multiplies plane hz by the stacked weights of q and
// writes from column (hz - 2) NT: its block n / NT = 1 - dz lands on output slice
// o = hz - 1 - dz, the one plane hz feeds through that z-tap, so every z-tap is summed
// in place.  Planes at the brick's z-ends feed fewer slices and use a narrower N (the
// part of the stack that lands inside [0, ZT NT)).  This makes (ZT + 2) x 9 MMAs of
// N up to 3 NT per input slice instead of ZT x 27 of N = NT: an MMA costs ~45 SM
// cycles whatever N up to 64, so for NT = 16 and 32 the tensor pipe does 2.4x fewer
// of them for the same work.  The MMAs of neighbouring planes add into shared
// columns, so one thread issues them all, in order, after the accumulators were
// zeroed with tcgen05.st, and commits them to the CTA's mbarrier once per slice.
// After the last slice the warps read the accumulators back (tcgen05.ld), add the
// bias, apply the ReLU and store bf16.
//
// ummaProbeKernel is the self-test of the inline-PTX interface in umma.cuh: one CTA
// stages A (128 x 16) and two B tiles (N x 16) in the no-swizzle K-major layout,
// issues three MMAs into two TMEM accumulators -- the first two sharing A through
// the A-operand collector (fill, lastuse), the third accumulating -- and reads the
// accumulators back.  Its buffer is laid out so that every access stays inside the
// 64 KB of shared memory it owns whichever stride of a descriptor is taken along K.
#include <algorithm>
#include <cstdint>

#include <cuda_runtime.h>

#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "denoiser.hpp"
#include "engine.hpp"
#include "umma.cuh"

namespace dxmcg {
namespace {

    constexpr int kProbeSmem = 64 * 1024;
    constexpr uint32_t kProbeA = 0;      // A: core (i, j) at i * 128 + j * 2048
    constexpr uint32_t kProbeB0 = 32768; // B: core (i, j) at i * 128 + j * 4096
    constexpr uint32_t kProbeB1 = 40960;
    constexpr uint32_t kWaitPolls = 1u << 22;

    __device__ __forceinline__ uint32_t coreOffset(int r, int k, uint32_t sbo, uint32_t lbo)
    {
        return static_cast<uint32_t>(r >> 3) * sbo + static_cast<uint32_t>(k >> 3) * lbo
            + static_cast<uint32_t>(r & 7) * 16u + static_cast<uint32_t>(k & 7) * 2u;
    }

    __global__ void __launch_bounds__(128) ummaProbeKernel(const uint16_t* __restrict__ A,
        const uint16_t* __restrict__ B0, const uint16_t* __restrict__ B1, int N, float* __restrict__ D0,
        float* __restrict__ D1, unsigned* __restrict__ status)
    {
        extern __shared__ __align__(128) unsigned char smem[];
        __shared__ __align__(8) uint64_t bar;
        __shared__ uint32_t tmemBase;
        const int t = threadIdx.x;
        const int warp = t >> 5;
        for (int e = t; e < 128 * 16; e += 128) {
            const int r = e >> 4, k = e & 15;
            *reinterpret_cast<uint16_t*>(smem + kProbeA + coreOffset(r, k, 128, 2048)) = A[e];
            if (r < N) {
                *reinterpret_cast<uint16_t*>(smem + kProbeB0 + coreOffset(r, k, 128, 4096)) = B0[e];
                *reinterpret_cast<uint16_t*>(smem + kProbeB1 + coreOffset(r, k, 128, 4096)) = B1[e];
            }
        }
        umma::fenceProxyAsync();
        if (warp == 0)
            umma::tmemAlloc(&tmemBase, 64);
        if (t == 0)
            umma::mbarInit(&bar, 1);
        umma::fenceBeforeSync();
        __syncthreads();
        umma::fenceAfterSync();
        const uint32_t tm = tmemBase;
        if (t == 0) {
            const uint32_t idesc = umma::instrDescriptorBf16(128, N);
            const uint32_t base = umma::smemAddr(smem);
            const uint64_t a = umma::smemDescriptor(base + kProbeA, 2048, 128);
            const uint64_t b0 = umma::smemDescriptor(base + kProbeB0, 4096, 128);
            const uint64_t b1 = umma::smemDescriptor(base + kProbeB1, 4096, 128);
            umma::mmaBf16<umma::Collector::kFill>(tm, a, b0, idesc, false);
            umma::mmaBf16<umma::Collector::kLastUse>(tm + 32, a, b1, idesc, false);
            umma::mmaBf16<umma::Collector::kNone>(tm, a, b1, idesc, true);
            umma::commit(&bar);
        }
        bool ok = umma::mbarWait(&bar, 0, kWaitPolls);
        if (!ok)
            ok = umma::mbarWait(&bar, 0, kWaitPolls); // a second bounded wait before touching TMEM
        umma::fenceAfterSync();
        const int row = 32 * warp + (t & 31);
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            umma::tmemLoad16(tm + (static_cast<uint32_t>(32 * warp) << 16) + c0, v);
            for (int i = 0; i < 16; ++i)
                D0[row * N + c0 + i] = v[i];
            umma::tmemLoad16(tm + (static_cast<uint32_t>(32 * warp) << 16) + 32 + c0, v);
            for (int i = 0; i < 16; ++i)
                D1[row * N + c0 + i] = v[i];
        }
        umma::fenceBeforeSync();
        __syncthreads();
        if (warp == 0) {
            umma::fenceAfterSync();
            umma::tmemFree(tm, 64);
        }
        if (t == 0) {
            if (!ok)
                atomicOr(status, 1u);
            umma::mbarInval(&bar);
        }
    }

    // ------------------------------------------------------------------ convolution
    __device__ unsigned g_convTcError; // set when a commit was not seen in time

    __device__ __forceinline__ void cpAsync16(uint32_t dst, const void* src, bool valid)
    {
        const int n = valid ? 16 : 0;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
    }

    template <int NT>
    struct ConvTcShape {
        static constexpr int ZT = NT == 64 ? 4 : 8;          // output z-slices per CTA
        static constexpr int HZ = ZT + 2, HY = 18, HX = 10;  // halo extent
        static constexpr int kVox = HZ * HY * HX;
        static constexpr uint32_t kPlane = kVox * 16;        // one 8-channel half of the halo
        static constexpr uint32_t kHalo = 2 * kPlane;
        static constexpr uint32_t kTapBytes = NT * 32;
        static constexpr uint32_t kStackBytes = 3 * kTapBytes; // the z-taps of one in-plane tap
        static constexpr uint32_t kWeights = 27 * kTapBytes;
        static constexpr uint32_t kSmem = kHalo + kWeights;
        static constexpr uint32_t kCols = ZT * NT <= 32 ? 32 : (ZT * NT <= 64 ? 64 : (ZT * NT <= 128 ? 128 : 256));
    };

    struct TcTile {
        int b, z0, y0, x0;
    };
    template <int ZT>
    __device__ __forceinline__ TcTile tcTileOf(int tile, int D, int H, int W)
    {
        const int nx = (W + 7) >> 3, ny = (H + 15) >> 4, nz = (D + ZT - 1) / ZT;
        TcTile p;
        p.x0 = (tile % nx) * 8;
        tile /= nx;
        p.y0 = (tile % ny) * 16;
        tile /= ny;
        p.z0 = (tile % nz) * ZT;
        p.b = tile / nz;
        return p;
    }

    // mapA / mapB: 5-D tensor maps (C, W, H, D, B) of the full-resolution inputs a and b
    // with a box of (8, 10, 18, ZT + 2, 1), used when useTma: the box of channel half h
    // lands as halo plane h.  Slices of an upsampled input (halfA) use cp.async.
    //
    // The CTAs are persistent: CTA (i, j) takes bricks i, i + gridDim.x, ... of output
    // channel tile j, keeping its TMEM, mbarriers and -- for a single 16-channel input
    // slice -- the weights for all of them (every brick reading the same weights from L2
    // made a few L2 slices the hot spot).  The epilogue zeroes the accumulators it read.
    template <int NT>
    __global__ void __launch_bounds__(256) conv3TcKernel(const nn::ConvIn in, int D, int H, int W, int Cin,
        const __nv_bfloat16* __restrict__ wgt, const float* __restrict__ bias, int Cout, int relu,
        __nv_bfloat16* __restrict__ out, const __grid_constant__ CUtensorMap mapA,
        const __grid_constant__ CUtensorMap mapB, int useTma, int tiles)
    {
        using S = ConvTcShape<NT>;
        constexpr int ZT = S::ZT;
        extern __shared__ __align__(128) unsigned char smem[];
        __shared__ __align__(8) uint64_t bar;
        __shared__ __align__(8) uint64_t tmaBar;
        __shared__ uint32_t tmemBase;
        const int t = threadIdx.x;
        const int warp = t >> 5;
        uint32_t tmaPhase = 0, mmaPhase = 0;
        const int n0 = blockIdx.y * NT;
        const int nSlices = Cin >> 4;
        const uint32_t sbase = umma::smemAddr(smem);
        const uint32_t wbase = sbase + S::kHalo;

        if (warp == 0)
            umma::tmemAlloc(&tmemBase, S::kCols);
        if (t == 0) {
            umma::mbarInit(&bar, 1);
            umma::mbarInit(&tmaBar, 1);
        }
        umma::fenceBeforeSync();
        __syncthreads();
        umma::fenceAfterSync();
        const uint32_t tm = tmemBase;
        const uint32_t laneBase = static_cast<uint32_t>(32 * (warp & 3)) << 16;
        // zero the accumulators (warp w: lanes 32 (w % 4).., half of the columns), so
        // that every MMA accumulates; the first slice's barrier orders these stores
        // before the MMAs
        {
            constexpr int half = ZT * NT / 2;
#pragma unroll
            for (int c = 0; c < half; c += 16)
                umma::tmemZero16(tm + laneBase + (warp >> 2) * half + c);
            umma::storeWait();
            umma::fenceBeforeSync();
        }
        // the slice's weights for all taps, z-taps stacked per in-plane tap (cp.async,
        // awaited with the halo of the slice)
        const auto stageWeights = [&](int c0) {
            for (int i = t; i < 27 * NT * 2; i += 256) {
                const int co = i % NT, th = i / NT; // th = tap * 2 + h, tap = 9 (dz + 1) + q
                const int tap = th >> 1, h = th & 1;
                const int dz1 = tap / 9, q = tap - 9 * dz1;
                const bool valid = n0 + co < Cout;
                const __nv_bfloat16* src
                    = valid ? wgt + ((static_cast<size_t>(n0 + co) * 27 + tap) * Cin + c0 + h * 8) : wgt;
                cpAsync16(wbase + q * S::kStackBytes + h * (3 * NT * 16) + ((2 - dz1) * NT + co) * 16, src, valid);
            }
        };
        const bool weightsResident = nSlices == 1;
        if (weightsResident)
            stageWeights(0);

        // 0: fine; kLateHalo / kLateMma: a bounded wait for the halo copies / the MMAs of
        // a slice gave up (the CTA stops, the device error flag is set)
        enum { kFine = 0, kLateHalo = 1, kLateMma = 2 };
        int failed = kFine;
        for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
            const TcTile p = tcTileOf<ZT>(tile, D, H, W);
            for (int sl = 0; sl < nSlices; ++sl) {
                const int c0 = sl * 16;
                // ---- stage the halo of this slice (from a, nearest-upsampled when halfA, or b)
                const bool inA = c0 < in.ca;
                const __nv_bfloat16* src = inA ? in.a : in.b;
                const int cs = inA ? in.ca : in.cb;
                const int cc = inA ? c0 : c0 - in.ca;
                const bool half = inA && in.halfA;
                const int Ds = half ? D >> 1 : D, Hs = half ? H >> 1 : H, Ws = half ? W >> 1 : W;
                // TMA needs a 128-byte aligned destination (checked here, not assumed)
                const bool tma = useTma && !half && (sbase & 127u) == 0u;
                if (tma && t == 0) {
                    const CUtensorMap* m = inA ? &mapA : &mapB;
                    umma::mbarArriveExpectTx(&tmaBar, S::kHalo);
                    umma::tmaLoad5d(sbase, m, cc, p.x0 - 1, p.y0 - 1, p.z0 - 1, p.b, &tmaBar);
                    umma::tmaLoad5d(sbase + S::kPlane, m, cc + 8, p.x0 - 1, p.y0 - 1, p.z0 - 1, p.b, &tmaBar);
                }
                for (int i = t; i < (tma ? 0 : 2 * S::kVox); i += 256) {
                    const int h = i / S::kVox, v = i - h * S::kVox;
                    const int hz = v / (S::HY * S::HX), hy = (v / S::HX) % S::HY, hx = v % S::HX;
                    const int gz = p.z0 + hz - 1, gy = p.y0 + hy - 1, gx = p.x0 + hx - 1;
                    const bool inside = gz >= 0 && gz < D && gy >= 0 && gy < H && gx >= 0 && gx < W;
                    const __nv_bfloat16* q = src;
                    if (inside) {
                        const int sz = half ? gz >> 1 : gz, sy = half ? gy >> 1 : gy, sx = half ? gx >> 1 : gx;
                        q = src + ((((static_cast<size_t>(p.b) * Ds + sz) * Hs + sy) * Ws + sx) * cs + cc + h * 8);
                    }
                    cpAsync16(sbase + h * S::kPlane + v * 16, q, inside);
                }
                if (!weightsResident)
                    stageWeights(c0);
                asm volatile("cp.async.commit_group;\n" ::);
                asm volatile("cp.async.wait_group 0;\n" ::: "memory");
                umma::fenceProxyAsync();
                int staged = 1;
                if (tma && t == 0)
                    staged = umma::mbarWait(&tmaBar, tmaPhase, 1u << 24) ? 1 : 0;
                if (!__syncthreads_and(staged)) {
                    failed = kLateHalo; // no MMAs were issued for this slice
                    break;
                }
                if (tma)
                    tmaPhase ^= 1u;

                // one thread issues the (ZT + 2) x 9 MMAs of the slice: plane hz feeds output
                // slices hz - dz1 for dz1 = dz + 1 in [lo, hi]; the stacked B rows of those
                // z-taps start at row (2 - hi) NT and land from column (hz - hi) NT
                if (t == 0) {
                    umma::fenceAfterSync();
                    // descriptor start addresses are in 16-byte units in the low 14 bits (shared
                    // memory < 256 KB), so offsets are added to the descriptor directly
                    const uint64_t aBase = umma::smemDescriptor(sbase, S::kPlane, S::HX * 16);
                    const uint64_t bBase = umma::smemDescriptor(wbase, 3 * NT * 16, 128);
                    // the plane loop stays rolled: unrolled, its 90-odd descriptors take ~170
                    // registers and cut the CTAs resident per SM from three to one
#pragma unroll 1
                    for (int hz = 0; hz < ZT + 2; ++hz) {
                        const int lo = hz - (ZT - 1) > 0 ? hz - (ZT - 1) : 0;
                        const int hi = hz < 2 ? hz : 2;
                        const uint32_t idesc = umma::instrDescriptorBf16(128, (hi - lo + 1) * NT);
                        const uint32_t d = tm + (hz - hi) * NT;
                        const uint64_t aPlane = aBase + static_cast<uint64_t>(hz * S::HY * S::HX);
                        const uint64_t bPlane = bBase + static_cast<uint64_t>(((2 - hi) * NT * 16) >> 4);
#pragma unroll
                        for (int q = 0; q < 9; ++q) {
                            const int dy1 = q / 3, dx1 = q % 3;
                            umma::mmaBf16<umma::Collector::kNone>(d,
                                aPlane + static_cast<uint64_t>(dy1 * S::HX + dx1),
                                bPlane + static_cast<uint64_t>((q * S::kStackBytes) >> 4), idesc, true);
                        }
                    }
                    umma::commit(&bar);
                }
                // the stage is free again (and, after the last slice, the sums are final)
                // once this slice's MMAs have completed: one thread polls the mbarrier, the
                // other warps wait at the CTA barrier without taking issue slots
                int done = 1;
                if (t == 0)
                    done = umma::mbarWait(&bar, mmaPhase, 1u << 24) ? 1 : 0;
                if (!__syncthreads_and(done)) {
                    failed = kLateMma;
                    break;
                }
                mmaPhase ^= 1u;
            }
            if (failed != kFine)
                break;
            umma::fenceAfterSync();

            // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows) for half the
            // slices, and zeroes what it read for the next brick
            const int lane = t & 31;
            const int row = 32 * (warp & 3) + lane;
            const int y = p.y0 + (row >> 3), x = p.x0 + (row & 7);
            const int oBegin = (warp >> 2) * (ZT / 2);
            const bool inPlane = y < H && x < W;
#pragma unroll 1
            for (int c = 0; c < NT; c += 16) {
                float bv[16];
#pragma unroll
                for (int k = 0; k < 16; ++k)
                    bv[k] = bias ? __ldg(bias + n0 + c + k) : 0.0f;
#pragma unroll 1
                for (int o = oBegin; o < oBegin + ZT / 2; ++o) {
                    float v[16];
                    const uint32_t ta = tm + laneBase + o * NT + c;
                    umma::tmemLoad16(ta, v);
                    umma::tmemZero16(ta);
                    const int z = p.z0 + o;
                    if (inPlane && z < D) {
                        uint4 pk[2];
                        __nv_bfloat162* h2 = reinterpret_cast<__nv_bfloat162*>(pk);
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            float a0 = v[2 * k] + bv[2 * k], a1 = v[2 * k + 1] + bv[2 * k + 1];
                            if (relu) {
                                a0 = fmaxf(a0, 0.0f);
                                a1 = fmaxf(a1, 0.0f);
                            }
                            h2[k] = __floats2bfloat162_rn(a0, a1);
                        }
                        uint4* d4 = reinterpret_cast<uint4*>(
                            out + (((static_cast<size_t>(p.b) * D + z) * H + y) * W + x) * Cout + n0 + c);
                        d4[0] = pk[0];
                        d4[1] = pk[1];
                    }
                }
            }
            // the zeros land before the next brick's MMAs (ordered by its first barrier)
            umma::storeWait();
            umma::fenceBeforeSync();
        }
        if (failed != kFine && t == 0) {
            atomicOr(&g_convTcError, 1u);
            // what is still in flight must land before the shared and tensor memory are
            // given back: the halo copies, or the MMAs, of the slice that gave up
            if (failed == kLateHalo)
                umma::mbarWait(&tmaBar, tmaPhase, 1u << 24);
            else
                umma::mbarWait(&bar, mmaPhase, 1u << 24);
        }
        // weights staged for a CTA that had no brick are awaited before it exits
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        umma::fenceBeforeSync();
        __syncthreads();
        if (warp == 0) {
            umma::fenceAfterSync();
            umma::tmemFree(tm, S::kCols);
        }
        if (t == 0) {
            umma::mbarInval(&bar);
            umma::mbarInval(&tmaBar);
        }
    }

    // cuTensorMapEncodeTiled from the driver, looked up once through the runtime
    PFN_cuTensorMapEncodeTiled_v12000 tensorMapEncoder()
    {
        static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
            void* p = nullptr;
            cudaDriverEntryPointQueryResult q {};
            if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q)
                    != cudaSuccess
                || q != cudaDriverEntryPointSuccess)
                p = nullptr;
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        }();
        return fn;
    }

    // 5-D map (C, W, H, D, B) of a channels-last bf16 tensor with a halo box
    // (8, 10, 18, hz, 1); false if it cannot be made (the kernel then uses cp.async)
    bool haloTensorMap(CUtensorMap* m, const void* base, int B, int D, int H, int W, int C, int hz)
    {
        const auto encode = tensorMapEncoder();
        if (!encode || !base || (reinterpret_cast<uintptr_t>(base) & 15u))
            return false;
        const cuuint64_t dims[5] = { static_cast<cuuint64_t>(C), static_cast<cuuint64_t>(W),
            static_cast<cuuint64_t>(H), static_cast<cuuint64_t>(D), static_cast<cuuint64_t>(B) };
        const cuuint64_t row = static_cast<cuuint64_t>(C) * 2;
        const cuuint64_t strides[4] = { row, row * W, row * W * H, row * W * H * D };
        const cuuint32_t box[5] = { 8, 10, 18, static_cast<cuuint32_t>(hz), 1 };
        const cuuint32_t step[5] = { 1, 1, 1, 1, 1 };
        return encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, step,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE)
            == CUDA_SUCCESS;
    }

    template <int NT>
    cudaError_t launchTc(const nn::ConvIn& in, int B, int D, int H, int W, int Cin, const __nv_bfloat16* w,
        const float* bias, int Cout, bool relu, __nv_bfloat16* out, cudaStream_t s)
    {
        using S = ConvTcShape<NT>;
        const int tiles = B * ((D + S::ZT - 1) / S::ZT) * ((H + 15) / 16) * ((W + 7) / 8);
        // tensor maps of the full-resolution inputs (an upsampled a keeps cp.async)
        CUtensorMap mapA {}, mapB {};
        bool tma = true;
        if (in.a && !in.halfA)
            tma = haloTensorMap(&mapA, in.a, B, D, H, W, in.ca, S::HZ);
        if (tma && in.b)
            tma = haloTensorMap(&mapB, in.b, B, D, H, W, in.cb, S::HZ);
        // persistent CTAs: as many as are resident at once (whole waves), never more than bricks
        // (from the SM's shared memory, registers and threads and the kernel's own use;
        // the occupancy query answered one CTA per SM where three are resident)
        static const int resident = [] {
            int dev = 0;
            cudaDeviceProp prop {};
            cudaFuncAttributes fa {};
            if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess
                || cudaFuncGetAttributes(&fa, conv3TcKernel<NT>) != cudaSuccess)
                return 0;
            const size_t perCta = S::kSmem + fa.sharedSizeBytes + prop.reservedSharedMemPerBlock;
            const int bySmem = static_cast<int>(prop.sharedMemPerMultiprocessor / perCta);
            const int regs = ((fa.numRegs + 7) / 8) * 8 * 256;
            const int byRegs = regs > 0 ? prop.regsPerMultiprocessor / regs : 1;
            const int byThreads = prop.maxThreadsPerMultiProcessor / 256;
            return std::max(1, std::min(bySmem, std::min(byRegs, byThreads))) * prop.multiProcessorCount;
        }();
        if (resident <= 0)
            return cudaErrorLaunchOutOfResources;
        const int gy = Cout / NT;
        const int gx = std::max(1, std::min(tiles, resident / gy));
        conv3TcKernel<NT><<<dim3(gx, gy), 256, S::kSmem, s>>>(in, D, H, W, Cin, w, bias, Cout, relu ? 1 : 0, out,
            mapA, mapB, tma ? 1 : 0, tiles);
        return cudaGetLastError();
    }

} // namespace

namespace nn {
    cudaError_t conv3TcConfigure()
    {
        // the whole unified L1 / shared array as shared memory: the CTAs per SM are
        // bounded by shared memory
        const auto configure = [](auto kernel, uint32_t smem) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                    cudaSharedmemCarveoutMaxShared);
            return e;
        };
        cudaError_t e = configure(conv3TcKernel<16>, ConvTcShape<16>::kSmem);
        if (e == cudaSuccess)
            e = configure(conv3TcKernel<32>, ConvTcShape<32>::kSmem);
        if (e == cudaSuccess)
            e = configure(conv3TcKernel<64>, ConvTcShape<64>::kSmem);
        return e;
    }

    cudaError_t launchConv3Tc(const ConvIn& in, int B, int D, int H, int W, int Cin, const __nv_bfloat16* w,
        const float* bias, int Cout, bool relu, __nv_bfloat16* out, cudaStream_t s)
    {
        if (Cin % 16 || Cout % 16 || (in.ca % 16) || (in.b && in.cb % 16) || in.ca + (in.b ? in.cb : 0) != Cin)
            return cudaErrorInvalidValue;
        if (Cout % 64 == 0)
            return launchTc<64>(in, B, D, H, W, Cin, w, bias, Cout, relu, out, s);
        if (Cout % 32 == 0)
            return launchTc<32>(in, B, D, H, W, Cin, w, bias, Cout, relu, out, s);
        return launchTc<16>(in, B, D, H, W, Cin, w, bias, Cout, relu, out, s);
    }

    int conv3TcCtas(int B, int D, int H, int W, int Cout)
    {
        const auto ctas = [&](int zt, int nt) {
            return B * ((D + zt - 1) / zt) * ((H + 15) / 16) * ((W + 7) / 8) * (Cout / nt);
        };
        if (Cout % 64 == 0)
            return ctas(ConvTcShape<64>::ZT, 64);
        if (Cout % 32 == 0)
            return ctas(ConvTcShape<32>::ZT, 32);
        return ctas(ConvTcShape<16>::ZT, 16);
    }

    // reads and clears the device flag of timed-out commits (0: none)
    cudaError_t conv3TcErrors(unsigned* flags)
    {
        unsigned zero = 0;
        cudaError_t e = cudaMemcpyFromSymbol(flags, g_convTcError, sizeof(unsigned));
        if (e == cudaSuccess && *flags)
            e = cudaMemcpyToSymbol(g_convTcError, &zero, sizeof(unsigned));
        return e;
    }
} // namespace nn

cudaError_t launchUmmaProbe(const uint16_t* A, const uint16_t* B0, const uint16_t* B1, int N, float* D0, float* D1,
    unsigned* status, cudaStream_t s)
{
    if (N != 16 && N != 32)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(ummaProbeKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kProbeSmem);
    if (e != cudaSuccess)
        return e;
    ummaProbeKernel<<<1, 128, kProbeSmem, s>>>(A, B0, B1, N, D0, D1, status);
    return cudaGetLastError();
}

} // namespace dxmcg
