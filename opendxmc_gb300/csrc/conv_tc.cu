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
        static constexpr int ZT = NT == 64 ? 4 : 8;          // output z-slices per brick
        static constexpr int HZ = ZT + 2, HY = 18, HX = 10;  // halo extent
        static constexpr int kVox = HZ * HY * HX;
        static constexpr uint32_t kPlane = kVox * 16;        // one 8-channel half of the halo
        static constexpr uint32_t kHalo = 2 * kPlane;        // one halo buffer (two in the pipeline)
        static constexpr uint32_t kTapBytes = NT * 32;
        static constexpr uint32_t kStackBytes = 3 * kTapBytes; // the z-taps of one in-plane tap
        static constexpr uint32_t kWeights = 27 * kTapBytes;  // one 16-channel input slice
        static constexpr uint32_t kAcc = ZT * NT;             // TMEM columns of one brick's sums
        static constexpr uint32_t kCols = 2 * kAcc <= 256 ? 256 : 512; // two accumulator sets
        // reach of a brick in a half-resolution input (nearest upsampling): low-resolution
        // voxels (z0/2 - 1 + lz, y0/2 - 1 + ly, x0/2 - 1 + lx), whose children cover the halo
        static constexpr int LZ = ZT / 2 + 2, LY = 10, LX = 6;
        static constexpr int kLowVox = LZ * LY * LX;
        // dynamic shared memory: one halo buffer per pipeline stage (two or three), then the
        // weights -- every slice's when they fit (resident), else one buffer per stage
        static constexpr int kMaxStages = 3;
        static constexpr uint32_t kMaxSmem = 227 * 1024 - 256;
        static constexpr uint32_t smemFor(int nSlices, bool resident, int stages)
        {
            return stages * kHalo + (resident ? nSlices : stages) * kWeights;
        }
        static_assert(2 * kHalo + 2 * kWeights <= kMaxSmem, "pipeline buffers exceed shared memory");
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
    // lands as halo plane h.  Slices of an upsampled input (halfA) are expanded by the
    // producer threads from the low-resolution voxels; without tensor maps the halo is
    // gathered with cp.async.
    //
    // One persistent CTA per SM (and output-channel tile blockIdx.y) works through its
    // items -- (brick, input slice) pairs, bricks blockIdx.x, blockIdx.x + gridDim.x, ...
    // in order, each brick's slices in order -- with warp-specialised roles that hand
    // work over through mbarriers only, never a CTA barrier:
    //   * warp 0 (one thread) issues each item's MMAs into its brick's accumulator set
    //     (the two sets alternate between bricks), commits them to empty[stage] and,
    //     after a brick's last slice, to accFull[set].  An issuing thread stalls while
    //     the tensor pipe's queue is full, so no other role waits on it;
    //   * warps 1-3 (producers) stage item i into stage i mod S once the MMAs of the
    //     item that used it before released it (S = 2 or 3 stages, a launch parameter):
    //     the halo by TMA (completing on tmaFull) or by their own
    //     copies / upsampling expansion, and the slice's weights unless every slice's
    //     weights stay resident; then they arrive on full[stage];
    //   * warps 4-7 (one TMEM lane quarter each) wait for accFull, read the brick's sums
    //     back (bias, ReLU, bf16 store), zero them and arrive on accEmpty[set].
    // Every wait is bounded; a role that gives up raises the CTA's abort flag, the
    // others leave at their next wait, and what is in flight (TMA, MMAs, copies) is
    // awaited before the shared and tensor memory are given back.
    constexpr int kProducers = 96;   // warps 1-3
    constexpr int kEpilogue = 128;   // warps 4-7
    constexpr uint32_t kPolls = 1u << 24;

    template <int NT>
    __global__ void __launch_bounds__(256, 1) conv3TcKernel(const nn::ConvIn in, int D, int H, int W, int Cin,
        const __nv_bfloat16* __restrict__ wgt, const float* __restrict__ bias, int Cout, int relu,
        __nv_bfloat16* __restrict__ out, const __grid_constant__ CUtensorMap mapA,
        const __grid_constant__ CUtensorMap mapB, int useTma, int tiles, int weightsResident, int stages,
        const nn::ConvOptions ep)
    {
        using S = ConvTcShape<NT>;
        constexpr int ZT = S::ZT;
        extern __shared__ __align__(128) unsigned char smem[];
        __shared__ __align__(8) uint64_t full[S::kMaxStages];    // producers' copies of stage b visible
        __shared__ __align__(8) uint64_t tmaFull[S::kMaxStages]; // the TMA halo of stage b landed
        __shared__ __align__(8) uint64_t empty[S::kMaxStages];   // the MMAs reading stage b are done
        __shared__ __align__(8) uint64_t accFull[2];  // the sums in accumulator set s are final
        __shared__ __align__(8) uint64_t accEmpty[2]; // set s was read back and zeroed
        __shared__ __align__(8) uint64_t drain;       // every MMA issued has completed
        __shared__ uint32_t tmemBase;
        __shared__ int abortFlag;
        const int t = threadIdx.x;
        const int warp = t >> 5;
        const int n0 = blockIdx.y * NT;
        const int nSlices = Cin >> 4;
        const uint32_t sbase = umma::smemAddr(smem);
        const uint32_t wbase = sbase + stages * S::kHalo;
        // this CTA's bricks: blockIdx.x, blockIdx.x + gridDim.x, ... of the brick list
        // (ep.list, ep.listLen entries) or of all `tiles` bricks
        const int nBricks = ep.list ? __ldg(ep.listLen) : tiles;
        const int myTiles = static_cast<int>(blockIdx.x) < nBricks
            ? (nBricks - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1
            : 0;
        const int nItems = myTiles * nSlices;
        volatile int* abortp = &abortFlag;
        // limit of the hand-over waits between the roles (the drains keep kPolls)
        const uint32_t hp = ep.handoverPolls ? ep.handoverPolls : kPolls;

        if (warp == 0)
            umma::tmemAlloc(&tmemBase, S::kCols);
        if (t == 0) {
            for (int b = 0; b < S::kMaxStages; ++b) {
                umma::mbarInit(&full[b], kProducers);
                umma::mbarInit(&tmaFull[b], 1);
                umma::mbarInit(&empty[b], 1);
            }
            for (int b = 0; b < 2; ++b) {
                umma::mbarInit(&accFull[b], 1);
                umma::mbarInit(&accEmpty[b], kEpilogue);
            }
            umma::mbarInit(&drain, 1);
            abortFlag = 0;
        }
        umma::fenceBeforeSync();
        __syncthreads();
        umma::fenceAfterSync();
        const uint32_t tm = tmemBase;
        const uint32_t laneBase = static_cast<uint32_t>(32 * (warp & 3)) << 16;
        // zero both accumulator sets (warp w: lanes 32 (w % 4).., half of the columns)
#pragma unroll
        for (int c = 0; c < static_cast<int>(S::kAcc); c += 16)
            umma::tmemZero16(tm + laneBase + (warp >> 2) * S::kAcc + c);
        umma::storeWait();

        // a slice's weights for all taps, z-taps stacked per in-plane tap (cp.async by the
        // threads [first, first + count))
        const auto stageWeights = [&](int sl, uint32_t dst, int first, int count) {
            const int c0 = sl * 16;
            for (int i = t - first; i < 27 * NT * 2; i += count) {
                const int co = i % NT, th = i / NT; // th = tap * 2 + h, tap = 9 (dz + 1) + q
                const int tap = th >> 1, h = th & 1;
                const int dz1 = tap / 9, q = tap - 9 * dz1;
                const bool valid = n0 + co < Cout;
                const __nv_bfloat16* src
                    = valid ? wgt + ((static_cast<size_t>(n0 + co) * 27 + tap) * Cin + c0 + h * 8) : wgt;
                cpAsync16(dst + q * S::kStackBytes + h * (3 * NT * 16) + ((2 - dz1) * NT + co) * 16, src, valid);
            }
        };
        if (weightsResident) {
            for (int sl = 0; sl < nSlices; ++sl)
                stageWeights(sl, wbase + sl * S::kWeights, 0, 256);
            asm volatile("cp.async.commit_group;\n" ::);
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        umma::fenceProxyAsync();
        umma::fenceBeforeSync();
        __syncthreads();
        umma::fenceAfterSync();

        const auto tileOfBrick = [&](int k) {
            const int j = static_cast<int>(blockIdx.x) + k * static_cast<int>(gridDim.x);
            return ep.list ? __ldg(ep.list + j) : j;
        };
        // whether the halo of slice sl comes by TMA (uniform over the CTA)
        const auto byTma = [&](int sl) {
            const bool inA = sl * 16 < in.ca;
            return useTma && !(inA && in.halfA) && (sbase & 127u) == 0u;
        };

        if (warp == 0) {
            // ------------------------------------------------------------ MMA issuer
            if (t == 0) {
                bool ok = true;
                uint32_t tmaPhase = 0; // bit b: phase of tmaFull[b] (only TMA items complete it)
                for (int it = 0; it < nItems && ok; ++it) {
                    const int b = it % stages;
                    const uint32_t use = static_cast<uint32_t>(it / stages);
                    const int sl = it % nSlices;
                    const int k = it / nSlices; // this CTA's brick number
                    const int set = k & 1;
                    ok = umma::mbarWaitOrAbort(&full[b], use & 1u, hp, abortp);
                    if (ok && byTma(sl)) {
                        ok = umma::mbarWaitOrAbort(&tmaFull[b], tmaPhase >> b & 1u, hp, abortp);
                        tmaPhase ^= 1u << b;
                    }
                    if (ok && sl == 0 && k >= 2)
                        ok = umma::mbarWaitOrAbort(&accEmpty[set], static_cast<uint32_t>((k >> 1) - 1) & 1u, hp,
                            abortp);
                    if (!ok)
                        break;
                    umma::fenceAfterSync();
                    // plane hz feeds output slices hz - dz1 for dz1 = dz + 1 in [lo, hi]; the
                    // stacked B rows of those z-taps start at row (2 - hi) NT and land from
                    // column (hz - hi) NT.  Descriptor start addresses are in 16-byte units in
                    // the low 14 bits (shared memory < 256 KB): offsets are added directly.
                    const uint64_t aBase = umma::smemDescriptor(sbase + b * S::kHalo, S::kPlane, S::HX * 16);
                    const uint64_t bBase = umma::smemDescriptor(
                        wbase + (weightsResident ? sl : b) * S::kWeights, 3 * NT * 16, 128);
                    const uint32_t dBase = tm + set * S::kAcc;
#pragma unroll 1
                    for (int hz = 0; hz < ZT + 2; ++hz) {
                        const int lo = hz - (ZT - 1) > 0 ? hz - (ZT - 1) : 0;
                        const int hi = hz < 2 ? hz : 2;
                        const uint32_t idesc = umma::instrDescriptorBf16(128, (hi - lo + 1) * NT);
                        const uint32_t d = dBase + (hz - hi) * NT;
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
                    umma::commit(&empty[b]);
                    if (sl == nSlices - 1)
                        umma::commit(&accFull[set]);
                }
                if (!ok)
                    *abortp = 1;
                // nothing issued may still run when the memory is given back
                umma::commit(&drain);
                if (!umma::mbarWait(&drain, 0, kPolls))
                    *abortp = 1;
            }
        } else if (warp < 4) {
            // ------------------------------------------------------------ producers
            const int pt = t - 32; // 0 .. kProducers - 1
            uint32_t tmaPending = 0, tmaPhase = 0;
            bool ok = true;
            for (int it = 0; it < nItems; ++it) {
                const int b = it % stages;
                const uint32_t use = static_cast<uint32_t>(it / stages);
                if (use >= 1 && !umma::mbarWaitOrAbort(&empty[b], (use - 1) & 1u, hp, abortp)) {
                    ok = false;
                    break;
                }
                if (pt == 0 && (tmaPending >> b & 1u)) {
                    // the stage's previous TMA was consumed by MMAs that are now done
                    tmaPending &= ~(1u << b);
                    tmaPhase ^= 1u << b;
                }
                const int sl = it % nSlices;
                const TcTile p = tcTileOf<ZT>(tileOfBrick(it / nSlices), D, H, W);
                const int c0 = sl * 16;
                const bool inA = c0 < in.ca;
                const __nv_bfloat16* src = inA ? in.a : in.b;
                const int cs = inA ? in.ca : in.cb;
                const int cc = inA ? c0 : c0 - in.ca;
                const bool half = inA && in.halfA;
                const uint32_t dst = sbase + b * S::kHalo;
                unsigned char* dstp = smem + b * S::kHalo;
                if (byTma(sl)) {
                    if (pt == 0) {
                        const CUtensorMap* m = inA ? &mapA : &mapB;
                        umma::mbarArriveExpectTx(&tmaFull[b], S::kHalo);
                        umma::tmaLoad5d(dst, m, cc, p.x0 - 1, p.y0 - 1, p.z0 - 1, p.b, &tmaFull[b]);
                        umma::tmaLoad5d(dst + S::kPlane, m, cc + 8, p.x0 - 1, p.y0 - 1, p.z0 - 1, p.b, &tmaFull[b]);
                        tmaPending |= 1u << b;
                    }
                } else if (half) {
                    // nearest upsampling: each low-resolution voxel of the brick's reach is
                    // read once and written to its 2 x 2 x 2 children that fall in the halo;
                    // with even dimensions a child is outside the volume exactly when its
                    // parent is, and that parent was read as zero
                    const int Ds = D >> 1, Hs = H >> 1, Ws = W >> 1;
                    constexpr int kBatch = 4;
                    for (int i0 = pt; i0 < 2 * S::kLowVox; i0 += kBatch * kProducers) {
                        uint4 lowv[kBatch];
#pragma unroll
                        for (int k = 0; k < kBatch; ++k) {
                            const int i = i0 + k * kProducers;
                            lowv[k] = make_uint4(0u, 0u, 0u, 0u);
                            if (i < 2 * S::kLowVox) {
                                const int h = i & 1, v = i >> 1;
                                const int lz = v / (S::LY * S::LX), ly = (v / S::LX) % S::LY, lx = v % S::LX;
                                const int sz = (p.z0 >> 1) - 1 + lz, sy = (p.y0 >> 1) - 1 + ly,
                                          sx = (p.x0 >> 1) - 1 + lx;
                                if (sz >= 0 && sz < Ds && sy >= 0 && sy < Hs && sx >= 0 && sx < Ws)
                                    lowv[k] = __ldg(reinterpret_cast<const uint4*>(src
                                        + ((((static_cast<size_t>(p.b) * Ds + sz) * Hs + sy) * Ws + sx) * cs + cc
                                            + h * 8)));
                            }
                        }
#pragma unroll
                        for (int k = 0; k < kBatch; ++k) {
                            const int i = i0 + k * kProducers;
                            if (i < 2 * S::kLowVox) {
                                const int h = i & 1, v = i >> 1;
                                const int lz = v / (S::LY * S::LX), ly = (v / S::LX) % S::LY, lx = v % S::LX;
                                // children at halo (2 lz - 1 + cz, ...): z0, y0 and x0 are even
                                const int hz0 = 2 * lz - 1, hy0 = 2 * ly - 1, hx0 = 2 * lx - 1;
                                unsigned char* base = dstp + h * S::kPlane;
#pragma unroll
                                for (int c = 0; c < 8; ++c) {
                                    const int hz = hz0 + (c >> 2), hy = hy0 + ((c >> 1) & 1), hx = hx0 + (c & 1);
                                    if (static_cast<unsigned>(hz) < static_cast<unsigned>(S::HZ)
                                        && static_cast<unsigned>(hy) < static_cast<unsigned>(S::HY)
                                        && static_cast<unsigned>(hx) < static_cast<unsigned>(S::HX))
                                        *reinterpret_cast<uint4*>(base + ((hz * S::HY + hy) * S::HX + hx) * 16)
                                            = lowv[k];
                                }
                            }
                        }
                    }
                } else {
                    // thread pairs copy the two 16-byte halves of one voxel: whole sectors
                    for (int i = pt; i < 2 * S::kVox; i += kProducers) {
                        const int h = i & 1, v = i >> 1;
                        const int hz = v / (S::HY * S::HX), hy = (v / S::HX) % S::HY, hx = v % S::HX;
                        const int gz = p.z0 + hz - 1, gy = p.y0 + hy - 1, gx = p.x0 + hx - 1;
                        const bool inside = gz >= 0 && gz < D && gy >= 0 && gy < H && gx >= 0 && gx < W;
                        const __nv_bfloat16* q = inside
                            ? src + ((((static_cast<size_t>(p.b) * D + gz) * H + gy) * W + gx) * cs + cc + h * 8)
                            : src;
                        cpAsync16(dst + h * S::kPlane + v * 16, q, inside);
                    }
                }
                if (!weightsResident)
                    stageWeights(sl, wbase + b * S::kWeights, 32, kProducers);
                asm volatile("cp.async.commit_group;\n" ::);
                asm volatile("cp.async.wait_group 0;\n" ::: "memory");
                umma::fenceProxyAsync(); // generic-proxy writes, read next by the tensor cores
                umma::mbarArrive(&full[b]);
            }
            if (!ok)
                *abortp = 1;
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
            // a TMA still in flight lands before the memory is given back
            if (pt == 0)
                for (int b = 0; b < stages; ++b)
                    if (tmaPending >> b & 1u)
                        umma::mbarWait(&tmaFull[b], tmaPhase >> b & 1u, kPolls);
        } else {
            // ------------------------------------------------------------ epilogue
            // per brick: bias, ReLU, bf16 store; with ep.pooled also the 2x2x2 averages
            // (z pairs in the thread, x pairs lane ^ 1, y pairs lane ^ 8: a warp holds 4
            // rows of 8 x); with ep.head (N_T = 16) the 1x1x1 head instead of the store
            const int lane = t & 31;
            const int row = 32 * (warp & 3) + lane;
            const bool pool = ep.pooled != nullptr;
            const bool head = NT == 16 && ep.head != nullptr;
            float hw[16];
            float hb = 0.0f;
#pragma unroll
            for (int j = 0; j < 16; ++j)
                hw[j] = head ? __ldg(ep.head + j) : 0.0f;
            if (head)
                hb = __ldg(ep.head + 16);
            const int Dh = D >> 1, Hh = H >> 1, Wh = W >> 1;
            for (int k = 0; k < myTiles; ++k) {
                const int set = k & 1;
                if (!umma::mbarWaitOrAbort(&accFull[set], static_cast<uint32_t>(k >> 1) & 1u, hp, abortp)) {
                    *abortp = 1;
                    break;
                }
                umma::fenceAfterSync();
                const TcTile p = tcTileOf<ZT>(tileOfBrick(k), D, H, W);
                const int y = p.y0 + (row >> 3), x = p.x0 + (row & 7);
                const bool inPlane = y < H && x < W;
                const uint32_t acc = tm + laneBase + set * S::kAcc;
#pragma unroll 1
                for (int c = 0; c < NT; c += 16) {
                    float bv[16];
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        bv[j] = bias ? __ldg(bias + n0 + c + j) : 0.0f;
#pragma unroll 1
                    for (int o = 0; o < ZT; o += 2) {
                        float r[2][16]; // the bf16 outputs of slices o and o + 1, as floats
#pragma unroll
                        for (int s2 = 0; s2 < 2; ++s2) {
                            float v[16];
                            const uint32_t ta = acc + (o + s2) * NT + c;
                            umma::tmemLoad16(ta, v);
                            umma::tmemZero16(ta);
                            uint4 pk[2];
                            __nv_bfloat162* h2 = reinterpret_cast<__nv_bfloat162*>(pk);
#pragma unroll
                            for (int j = 0; j < 8; ++j) {
                                float a0 = v[2 * j] + bv[2 * j], a1 = v[2 * j + 1] + bv[2 * j + 1];
                                if (relu) {
                                    a0 = fmaxf(a0, 0.0f);
                                    a1 = fmaxf(a1, 0.0f);
                                }
                                h2[j] = __floats2bfloat162_rn(a0, a1);
                                const float2 f = __bfloat1622float2(h2[j]);
                                r[s2][2 * j] = f.x;
                                r[s2][2 * j + 1] = f.y;
                            }
                            const int z = p.z0 + o + s2;
                            if (inPlane && z < D) {
                                const size_t vox = ((static_cast<size_t>(p.b) * D + z) * H + y) * W + x;
                                if (head) {
                                    float pr = hb;
#pragma unroll
                                    for (int j = 0; j < 16; ++j)
                                        pr = fmaf(r[s2][j], hw[j], pr);
                                    if (ep.headPred)
                                        ep.headPred[vox] = pr;
                                    if (ep.headOut)
                                        ep.headOut[vox] = static_cast<double>(pr) * ep.headScale;
                                } else {
                                    uint4* d4 = reinterpret_cast<uint4*>(out + vox * Cout + n0 + c);
                                    d4[0] = pk[0];
                                    d4[1] = pk[1];
                                }
                            }
                        }
                        if (pool) {
                            float sum[16];
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                sum[j] = r[0][j] + r[1][j];
                                sum[j] += __shfl_xor_sync(0xffffffffu, sum[j], 1);
                                sum[j] += __shfl_xor_sync(0xffffffffu, sum[j], 8);
                            }
                            // the even corner writes; with even D, H, W its window is inside
                            // the volume exactly when the corner is
                            if ((lane & 9) == 0 && inPlane && p.z0 + o < D) {
                                uint4 pk[2];
                                __nv_bfloat162* h2 = reinterpret_cast<__nv_bfloat162*>(pk);
#pragma unroll
                                for (int j = 0; j < 8; ++j)
                                    h2[j] = __floats2bfloat162_rn(sum[2 * j] * 0.125f, sum[2 * j + 1] * 0.125f);
                                uint4* d4 = reinterpret_cast<uint4*>(ep.pooled
                                    + ((((static_cast<size_t>(p.b) * Dh + ((p.z0 + o) >> 1)) * Hh + (y >> 1)) * Wh
                                           + (x >> 1))
                                              * Cout
                                        + n0 + c));
                                d4[0] = pk[0];
                                d4[1] = pk[1];
                            }
                        }
                    }
                }
                // the zeros land before the set's next MMAs
                umma::storeWait();
                umma::fenceBeforeSync();
                umma::mbarArrive(&accEmpty[set]);
            }
        }

        umma::fenceBeforeSync();
        __syncthreads();
        if (t == 0 && abortFlag)
            atomicOr(&g_convTcError, 1u);
        if (warp == 0) {
            umma::fenceAfterSync();
            umma::tmemFree(tm, S::kCols);
        }
        if (t == 0) {
            for (int b = 0; b < S::kMaxStages; ++b) {
                umma::mbarInval(&full[b]);
                umma::mbarInval(&tmaFull[b]);
                umma::mbarInval(&empty[b]);
            }
            for (int b = 0; b < 2; ++b) {
                umma::mbarInval(&accFull[b]);
                umma::mbarInval(&accEmpty[b]);
            }
            umma::mbarInval(&drain);
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
        const float* bias, int Cout, bool relu, __nv_bfloat16* out, cudaStream_t s, const nn::ConvOptions& ep)
    {
        using S = ConvTcShape<NT>;
        const int tiles = B * ((D + S::ZT - 1) / S::ZT) * ((H + 15) / 16) * ((W + 7) / 8);
        // tensor maps of the full-resolution inputs (an upsampled a is expanded by the threads)
        CUtensorMap mapA {}, mapB {};
        bool tma = true;
        if (in.a && !in.halfA)
            tma = haloTensorMap(&mapA, in.a, B, D, H, W, in.ca, S::HZ);
        if (tma && in.b)
            tma = haloTensorMap(&mapB, in.b, B, D, H, W, in.cb, S::HZ);
        // one persistent CTA per SM and output-channel tile, never more than bricks
        static const int sms = [] {
            int dev = 0, n = 0;
            if (cudaGetDevice(&dev) != cudaSuccess
                || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
                return 0;
            return n;
        }();
        if (sms <= 0)
            return cudaErrorLaunchOutOfResources;
        const int nSlices = Cin / 16;
        // resident weights where they fit; two stages (a third, where it fits, measured no
        // faster on the 512 x 512 x 400 inference: the tensor pipe, not the staging, is the
        // bound)
        const bool resident = S::smemFor(nSlices, true, 2) <= S::kMaxSmem;
        const int stages = 2;
        const int gy = Cout / NT;
        const int gx = std::max(1, std::min(tiles, sms / gy));
        conv3TcKernel<NT><<<dim3(gx, gy), 256, S::smemFor(nSlices, resident, stages), s>>>(in, D, H, W, Cin, w, bias,
            Cout, relu ? 1 : 0, out, mapA, mapB, tma ? 1 : 0, tiles, resident ? 1 : 0, stages, ep);
        return cudaGetLastError();
    }

    // For each job j (one CTA of 1024 threads each): list_j[0 .. *len_j) = the indices b
    // with mask_j[b] != 0, in increasing order.  A pass covers 4096 bricks, four
    // consecutive ones per thread: counts scanned within warps, a prefix over the warps.
    __global__ void __launch_bounds__(1024) brickListKernel(const nn::BrickListJobs jobs)
    {
        __shared__ int warpBase[32];
        __shared__ int passTotal;
        const int j = static_cast<int>(blockIdx.x);
        const uint8_t* __restrict__ active = jobs.mask[j];
        int* __restrict__ list = jobs.list[j];
        const int nb = jobs.nb[j];
        const bool words = (reinterpret_cast<uintptr_t>(active) & 3u) == 0u;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        int base = 0;
        for (int i0 = 0; i0 < nb; i0 += 4096) {
            const int i = i0 + 4 * static_cast<int>(threadIdx.x);
            unsigned f = 0; // bit k: brick i + k is marked
            if (words && i + 3 < nb) {
                const uchar4 v = *reinterpret_cast<const uchar4*>(active + i);
                f = (v.x != 0 ? 1u : 0u) | (v.y != 0 ? 2u : 0u) | (v.z != 0 ? 4u : 0u) | (v.w != 0 ? 8u : 0u);
            } else {
                for (int k = 0; k < 4; ++k)
                    if (i + k < nb && active[i + k] != 0)
                        f |= 1u << k;
            }
            const int c = __popc(f);
            int incl = c;
            for (int o = 1; o < 32; o <<= 1) {
                const int n = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                    incl += n;
            }
            if (lane == 31)
                warpBase[w] = incl;
            __syncthreads();
            if (w == 0) {
                const int v = warpBase[lane];
                int sum = v;
                for (int o = 1; o < 32; o <<= 1) {
                    const int n = __shfl_up_sync(0xffffffffu, sum, o);
                    if (lane >= o)
                        sum += n;
                }
                warpBase[lane] = sum - v;
                if (lane == 31)
                    passTotal = sum;
            }
            __syncthreads();
            int pos = base + warpBase[w] + incl - c;
            for (int k = 0; k < 4; ++k)
                if (f >> k & 1u)
                    list[pos++] = i + k;
            base += passTotal;
            __syncthreads(); // warpBase and passTotal are rewritten by the next pass
        }
        if (threadIdx.x == 0)
            *jobs.len[j] = base;
    }

    // grown[b] = 1 where brick b or one of its 26 neighbours is active
    __global__ void brickGrowKernel(const uint8_t* __restrict__ active, int cx, int cy, int cz,
        uint8_t* __restrict__ grown)
    {
        const int nb = cx * cy * cz;
        for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
            const int ix = b % cx, iy = (b / cx) % cy, iz = b / (cx * cy);
            uint8_t g = 0;
            for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        const int x = ix + dx, y = iy + dy, z = iz + dz;
                        if (x >= 0 && x < cx && y >= 0 && y < cy && z >= 0 && z < cz)
                            g |= active[(static_cast<size_t>(z) * cy + y) * cx + x];
                    }
            grown[b] = g;
        }
    }

    // One pass of a separable union of brick boxes: `out` has in's counts (nx, ny, nz)
    // with the count along `axis` (0: x, 1: y, 2: z) replaced by nOut, and out[.., b, ..]
    // = 1 where in[.., c, ..] is marked for some c in [range[2b], range[2b + 1]].
    __global__ void brickMapAxisKernel(const uint8_t* __restrict__ in, int nx, int ny, int nz, int axis, int nOut,
        const int* __restrict__ range, uint8_t* __restrict__ out)
    {
        const int ox = axis == 0 ? nOut : nx, oy = axis == 1 ? nOut : ny, oz = axis == 2 ? nOut : nz;
        const int total = ox * oy * oz;
        for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < total; o += gridDim.x * blockDim.x) {
            const int x = o % ox, y = (o / ox) % oy, z = o / (ox * oy);
            const int b = axis == 0 ? x : (axis == 1 ? y : z);
            const int c1 = range[2 * b + 1];
            uint8_t v = 0;
            for (int c = range[2 * b]; c <= c1 && !v; ++c) {
                const int ix = axis == 0 ? c : x, iy = axis == 1 ? c : y, iz = axis == 2 ? c : z;
                v = in[(static_cast<size_t>(iz) * ny + iy) * nx + ix];
            }
            out[o] = v ? 1 : 0;
        }
    }


} // namespace

namespace nn {
    cudaError_t conv3TcConfigure()
    {
        // the whole unified L1 / shared array as shared memory (one CTA per SM, with up to
        // ConvTcShape::kMaxSmem of pipeline buffers)
        const auto configure = [](auto kernel, uint32_t smem) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                    cudaSharedmemCarveoutMaxShared);
            return e;
        };
        cudaError_t e = configure(conv3TcKernel<16>, ConvTcShape<16>::kMaxSmem);
        if (e == cudaSuccess)
            e = configure(conv3TcKernel<32>, ConvTcShape<32>::kMaxSmem);
        if (e == cudaSuccess)
            e = configure(conv3TcKernel<64>, ConvTcShape<64>::kMaxSmem);
        return e;
    }

    cudaError_t launchConv3Tc(const ConvIn& in, int B, int D, int H, int W, int Cin, const __nv_bfloat16* w,
        const float* bias, int Cout, bool relu, __nv_bfloat16* out, cudaStream_t s, const ConvOptions* ep)
    {
        if (Cin % 16 || Cout % 16 || (in.ca % 16) || (in.b && in.cb % 16) || in.ca + (in.b ? in.cb : 0) != Cin)
            return cudaErrorInvalidValue;
        const ConvOptions none {};
        const ConvOptions& e = ep ? *ep : none;
        // the pooled output needs whole 2 x 2 x 2 windows; the head a 16-channel output
        if ((e.pooled && ((D | H | W) & 1)) || (e.head && Cout != 16))
            return cudaErrorInvalidValue;
        if (Cout % 64 == 0)
            return launchTc<64>(in, B, D, H, W, Cin, w, bias, Cout, relu, out, s, e);
        if (Cout % 32 == 0)
            return launchTc<32>(in, B, D, H, W, Cin, w, bias, Cout, relu, out, s, e);
        return launchTc<16>(in, B, D, H, W, Cin, w, bias, Cout, relu, out, s, e);
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

    void conv3TcBrickDims(int D, int H, int W, int Cout, int brick[3], int count[3])
    {
        const int zt = Cout % 64 == 0 ? ConvTcShape<64>::ZT : (Cout % 32 == 0 ? ConvTcShape<32>::ZT : ConvTcShape<16>::ZT);
        brick[0] = 8;
        brick[1] = 16;
        brick[2] = zt;
        count[0] = (W + 7) / 8;
        count[1] = (H + 15) / 16;
        count[2] = (D + zt - 1) / zt;
    }

    cudaError_t launchBrickGrow(const uint8_t* active, const int count[3], uint8_t* grown, cudaStream_t s)
    {
        const int nb = count[0] * count[1] * count[2];
        brickGrowKernel<<<std::max(1, std::min((nb + 255) / 256, 4096)), 256, 0, s>>>(active, count[0], count[1],
            count[2], grown);
        return cudaGetLastError();
    }

    cudaError_t launchBrickMap(const uint8_t* in, const int inCount[3], const int outCount[3], const int* ranges,
        uint8_t* out, uint8_t* tmp1, uint8_t* tmp2, cudaStream_t s)
    {
        for (int a = 0; a < 3; ++a)
            if (inCount[a] < 1 || outCount[a] < 1)
                return cudaErrorInvalidValue;
        if (!in || !ranges || !out || !tmp1 || !tmp2 || in == out || in == tmp1 || in == tmp2 || out == tmp1
            || out == tmp2 || tmp1 == tmp2)
            return cudaErrorInvalidValue;
        const auto grid = [](int items) { return std::max(1, std::min((items + 255) / 256, 4096)); };
        const int* rx = ranges;
        const int* ry = rx + 2 * outCount[0];
        const int* rz = ry + 2 * outCount[1];
        brickMapAxisKernel<<<grid(outCount[0] * inCount[1] * inCount[2]), 256, 0, s>>>(in, inCount[0], inCount[1],
            inCount[2], 0, outCount[0], rx, tmp1);
        brickMapAxisKernel<<<grid(outCount[0] * outCount[1] * inCount[2]), 256, 0, s>>>(tmp1, outCount[0],
            inCount[1], inCount[2], 1, outCount[1], ry, tmp2);
        brickMapAxisKernel<<<grid(outCount[0] * outCount[1] * outCount[2]), 256, 0, s>>>(tmp2, outCount[0],
            outCount[1], inCount[2], 2, outCount[2], rz, out);
        return cudaGetLastError();
    }

    cudaError_t launchBrickLists(const BrickListJobs& jobs, cudaStream_t s)
    {
        if (jobs.n < 1 || jobs.n > kMaxBrickLists)
            return cudaErrorInvalidValue;
        for (int j = 0; j < jobs.n; ++j)
            if (!jobs.mask[j] || !jobs.list[j] || !jobs.len[j] || jobs.nb[j] < 0)
                return cudaErrorInvalidValue;
        brickListKernel<<<jobs.n, 1024, 0, s>>>(jobs);
        return cudaGetLastError();
    }

    cudaError_t launchBrickList(const uint8_t* mask, int nb, int* list, int* listLen, cudaStream_t s)
    {
        BrickListJobs jobs;
        jobs.add(mask, nb, list, listLen);
        return launchBrickLists(jobs, s);
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
