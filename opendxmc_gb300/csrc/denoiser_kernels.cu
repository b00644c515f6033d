// denoiser_kernels.cu -- kernels of the dose denoiser (a 3D convolutional
// encoder-decoder trained on the transport's own low/high-history dose pairs).
// This part has no counterpart in the reference.
//
// Tensors are [B][D][H][W][C] bfloat16 with C a multiple of 16 ("channels last"),
// so that 16 channels of one voxel are one 32-byte row.  A 3x3x3 convolution is an
// implicit GEMM: rows = output voxels, columns = output channels, reduction =
// 27 taps x input channels.  A CTA owns an 8x8x8 brick of output voxels and
// NT output channels; per 16-channel slice of the input it stages the 10x10x10
// halo brick and the slice's weights in shared memory (cp.async, double
// buffered), and every tap then reads the same halo brick shifted by one voxel:
// each input element is fetched from global memory once per CTA instead of 27
// times.  The products run on the tensor cores as bf16 mma.sync m16n8k16 with
// FP32 accumulation; rows are loaded with ldmatrix from shared memory whose
// 16-byte halves are XOR-swizzled so that the eight rows of a matrix fall in
// distinct banks.
#include <cstdint>

#include <cuda_bf16.h>

#include "denoiser.hpp"

namespace dxmcg {
namespace nn {
namespace {

    constexpr int kHaloVox = 1000;            // 10 x 10 x 10
    constexpr int kHaloBytes = kHaloVox * 32; // 16 channels of bf16 per voxel

    __device__ __forceinline__ unsigned smemAddr(const void* p)
    {
        return static_cast<unsigned>(__cvta_generic_to_shared(p));
    }

    // 16-byte asynchronous copy global -> shared; zero fill when !valid (no read)
    __device__ __forceinline__ void cpAsync16(unsigned dst, const void* src, bool valid)
    {
        const int n = valid ? 16 : 0;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
    }
    __device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::); }
    template <int N>
    __device__ __forceinline__ void cpAsyncWait()
    {
        asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
    }

    __device__ __forceinline__ void ldsm4(unsigned addr, unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3)
    {
        asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                     : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                     : "r"(addr));
    }
    __device__ __forceinline__ void ldsm4t(unsigned addr, unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3)
    {
        asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                     : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                     : "r"(addr));
    }
    // D = A (16x16, row) * B (16x8, col) + D, bf16 inputs, f32 accumulators
    __device__ __forceinline__ void mma16816(float (&c)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
        unsigned b0, unsigned b1)
    {
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                     "{%0,%1,%2,%3};\n"
                     : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                     : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }

    __device__ __forceinline__ int tapDz(int t) { return t / 9 - 1; }
    __device__ __forceinline__ int tapDy(int t) { return (t / 3) % 3 - 1; }
    __device__ __forceinline__ int tapDx(int t) { return t % 3 - 1; }

    struct BrickPos {
        int b, z0, y0, x0;
    };
    __device__ __forceinline__ BrickPos brickOf(int brick, int D, int H, int W)
    {
        const int nbx = (W + 7) >> 3, nby = (H + 7) >> 3, nbz = (D + 7) >> 3;
        BrickPos p;
        p.x0 = (brick % nbx) * 8;
        brick /= nbx;
        p.y0 = (brick % nby) * 8;
        brick /= nby;
        p.z0 = (brick % nbz) * 8;
        p.b = brick / nbz;
        return p;
    }

    // Stage the halo brick of one 16-channel input slice: halo voxel v = (hz*10 + hy)*10
    // + hx holds its two 16-byte halves at v*32 + ((h ^ ((hx >> 2) & 1)) << 4).
    __device__ __forceinline__ void loadHalo(const ConvIn& in, int c0, const BrickPos& p, int D, int H, int W,
        unsigned sbase)
    {
        const bool inA = c0 < in.ca;
        const __nv_bfloat16* src = inA ? in.a : in.b;
        const int cs = inA ? in.ca : in.cb;
        const int cc = inA ? c0 : c0 - in.ca;
        const bool half = inA && in.halfA;
        const int Ds = half ? D >> 1 : D, Hs = half ? H >> 1 : H, Ws = half ? W >> 1 : W;
        for (int i = threadIdx.x; i < 2 * kHaloVox; i += blockDim.x) {
            const int v = i >> 1, h = i & 1;
            const int hz = v / 100, hy = (v / 10) % 10, hx = v % 10;
            const int gz = p.z0 + hz - 1, gy = p.y0 + hy - 1, gx = p.x0 + hx - 1;
            const bool ok = gz >= 0 && gz < D && gy >= 0 && gy < H && gx >= 0 && gx < W;
            const __nv_bfloat16* q = src;
            if (ok) {
                const int sz = half ? gz >> 1 : gz, sy = half ? gy >> 1 : gy, sx = half ? gx >> 1 : gx;
                q = src + ((((static_cast<size_t>(p.b) * Ds + sz) * Hs + sy) * Ws + sx) * cs + cc + h * 8);
            }
            cpAsync16(sbase + v * 32 + ((h ^ ((hx >> 2) & 1)) << 4), q, ok);
        }
    }

    // ------------------------------------------------------------------ forward conv
    template <int NT>
    __global__ void __launch_bounds__(256, 1) conv3Kernel(const ConvIn in, int D, int H, int W, int Cin,
        const __nv_bfloat16* __restrict__ wgt, const float* __restrict__ bias, int Cout, int relu,
        __nv_bfloat16* __restrict__ out)
    {
        extern __shared__ __align__(128) unsigned char smem[];
        constexpr int kWBytes = 27 * NT * 32;
        constexpr int kStage = kHaloBytes + kWBytes;
        const BrickPos p = brickOf(blockIdx.x, D, H, W);
        const int n0 = blockIdx.y * NT;
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int nChunks = Cin >> 4;

        auto load = [&](int chunk, int stage) {
            const unsigned sbase = smemAddr(smem + stage * kStage);
            const int c0 = chunk * 16;
            loadHalo(in, c0, p, D, H, W, sbase);
            const unsigned wbase = sbase + kHaloBytes;
            for (int i = threadIdx.x; i < 27 * NT * 2; i += blockDim.x) {
                const int h = i & 1, row = i >> 1; // row = tap * NT + co
                const int tap = row / NT, co = row % NT;
                const bool ok = n0 + co < Cout;
                const __nv_bfloat16* q
                    = ok ? wgt + ((static_cast<size_t>(n0 + co) * 27 + tap) * Cin + c0 + h * 8) : wgt;
                cpAsync16(wbase + row * 32 + ((h ^ ((co >> 2) & 1)) << 4), q, ok);
            }
            cpAsyncCommit();
        };

        float acc[4][NT / 8][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < NT / 8; ++j)
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    acc[i][j][k] = 0.0f;

        const int q = lane >> 3, r = lane & 7;
        load(0, 0);
        for (int chunk = 0; chunk < nChunks; ++chunk) {
            if (chunk + 1 < nChunks) {
                load(chunk + 1, (chunk + 1) & 1);
                cpAsyncWait<1>();
            } else {
                cpAsyncWait<0>();
            }
            __syncthreads();
            const unsigned sbase = smemAddr(smem + (chunk & 1) * kStage);
            const unsigned wbase = sbase + kHaloBytes;
#pragma unroll 1
            for (int tap = 0; tap < 27; ++tap) {
                const int dz = tapDz(tap), dy = tapDy(tap), dx = tapDx(tap);
                unsigned bf[NT / 8][2];
#pragma unroll
                for (int j = 0; j < NT / 16; ++j) {
                    const int co = j * 16 + ((q >> 1) << 3) + r;
                    const int h = q & 1;
                    ldsm4(wbase + (tap * NT + co) * 32 + ((h ^ ((co >> 2) & 1)) << 4), bf[2 * j][0], bf[2 * j][1],
                        bf[2 * j + 1][0], bf[2 * j + 1][1]);
                }
                const int hz = warp + dz + 1, hx = r + dx + 1;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int hy = 2 * i + (q & 1) + dy + 1;
                    const int v = (hz * 10 + hy) * 10 + hx;
                    const int h = q >> 1;
                    unsigned a0, a1, a2, a3;
                    ldsm4(sbase + v * 32 + ((h ^ ((hx >> 2) & 1)) << 4), a0, a1, a2, a3);
#pragma unroll
                    for (int j = 0; j < NT / 8; ++j)
                        mma16816(acc[i][j], a0, a1, a2, a3, bf[j][0], bf[j][1]);
                }
            }
            __syncthreads(); // the next iteration's load reuses this stage
        }

        const int g = lane >> 2, t = lane & 3;
        const int z = p.z0 + warp;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
                const int y = p.y0 + 2 * i + hf, x = p.x0 + g;
                if (z >= D || y >= H || x >= W)
                    continue;
                __nv_bfloat16* o = out + (((static_cast<size_t>(p.b) * D + z) * H + y) * W + x) * Cout;
#pragma unroll
                for (int j = 0; j < NT / 8; ++j) {
                    const int co = n0 + 8 * j + 2 * t;
                    if (co >= Cout)
                        continue;
                    float v0 = acc[i][j][2 * hf], v1 = acc[i][j][2 * hf + 1];
                    if (bias) {
                        v0 += bias[co];
                        v1 += bias[co + 1];
                    }
                    if (relu) {
                        v0 = fmaxf(v0, 0.0f);
                        v1 = fmaxf(v1, 0.0f);
                    }
                    *reinterpret_cast<__nv_bfloat162*>(o + co) = __floats2bfloat162_rn(v0, v1);
                }
            }
    }

    // ------------------------------------------------------------------ weight gradient
    // dW[co][tap][ci] += sum over output voxels v of dz[v][co] * x[v + off(tap)][ci].
    // grid: x = CTAs looping over bricks, y = output-channel tile, z = input slice.
    // Warp w owns taps w, w+8, w+16 (and 24 for w < 3) and keeps their partial sums
    // in registers across all its bricks; one atomic flush per CTA at the end.
    template <int NT>
    __global__ void __launch_bounds__(256, 1) wgradKernel(const ConvIn in, const __nv_bfloat16* __restrict__ dz,
        int D, int H, int W, int Cin, int Cout, int nBricks, float* __restrict__ dW)
    {
        extern __shared__ __align__(128) unsigned char smem[];
        constexpr int kRow = NT * 2; // bytes of one voxel's NT gradient values
        constexpr int kChunks = NT / 8;
        const unsigned haloBase = smemAddr(smem);
        const unsigned dzBase = haloBase + kHaloBytes;
        const int n0 = blockIdx.y * NT;
        const int c0 = blockIdx.z * 16;
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int q = lane >> 3, r = lane & 7;
        const int nSlots = warp < 3 ? 4 : 3;

        float acc[4][NT / 16][2][4];
#pragma unroll
        for (int s = 0; s < 4; ++s)
#pragma unroll
            for (int m = 0; m < NT / 16; ++m)
#pragma unroll
                for (int n = 0; n < 2; ++n)
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        acc[s][m][n][k] = 0.0f;

        for (int brick = blockIdx.x; brick < nBricks; brick += gridDim.x) {
            const BrickPos p = brickOf(brick, D, H, W);
            loadHalo(in, c0, p, D, H, W, haloBase);
            for (int i = threadIdx.x; i < 512 * kChunks; i += blockDim.x) {
                const int v = i / kChunks, c = i % kChunks;
                const int z = p.z0 + (v >> 6), y = p.y0 + ((v >> 3) & 7), x = p.x0 + (v & 7);
                const bool ok = z < D && y < H && x < W;
                const __nv_bfloat16* src
                    = ok ? dz + ((((static_cast<size_t>(p.b) * D + z) * H + y) * W + x) * Cout + n0 + c * 8) : dz;
                const int key = NT == 32 ? ((v >> 1) & 3) : ((v >> 2) & 1);
                cpAsync16(dzBase + v * kRow + ((c ^ key) << 4), src, ok);
            }
            cpAsyncCommit();
            cpAsyncWait<0>();
            __syncthreads();
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                if (s >= nSlots)
                    break;
                const int tap = warp + 8 * s;
                const int dzt = tapDz(tap), dyt = tapDy(tap), dxt = tapDx(tap);
#pragma unroll 2
                for (int ks = 0; ks < 32; ++ks) {
                    // voxels 16 ks .. 16 ks + 15 of the brick: z = ks / 4, y = 2 (ks % 4) + (row >= 8)
                    const int zz = ks >> 2, yb = (ks & 3) * 2;
                    // B: x rows (k = voxel), 8 input channels per matrix, transposed
                    unsigned b00, b01, b10, b11;
                    {
                        const int yy = yb + (q & 1);
                        const int hz = zz + dzt + 1, hy = yy + dyt + 1, hx = r + dxt + 1;
                        const int v = (hz * 10 + hy) * 10 + hx;
                        const int h = q >> 1;
                        ldsm4t(haloBase + v * 32 + ((h ^ ((hx >> 2) & 1)) << 4), b00, b01, b10, b11);
                    }
#pragma unroll
                    for (int m = 0; m < NT / 16; ++m) {
                        // A: dz rows (k = voxel) x 8 output channels per matrix, transposed
                        const int vrow = ks * 16 + ((q >> 1) << 3) + r;
                        const int c = m * 2 + (q & 1);
                        const int key = NT == 32 ? ((vrow >> 1) & 3) : ((vrow >> 2) & 1);
                        unsigned a0, a1, a2, a3;
                        ldsm4t(dzBase + vrow * kRow + ((c ^ key) << 4), a0, a1, a2, a3);
                        mma16816(acc[s][m][0], a0, a1, a2, a3, b00, b01);
                        mma16816(acc[s][m][1], a0, a1, a2, a3, b10, b11);
                    }
                }
            }
            __syncthreads(); // the next brick's loads overwrite the staging
        }

        const int g = lane >> 2, t = lane & 3;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            if (s >= nSlots)
                break;
            const int tap = warp + 8 * s;
#pragma unroll
            for (int m = 0; m < NT / 16; ++m)
#pragma unroll
                for (int n = 0; n < 2; ++n)
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int co = n0 + m * 16 + g + ((k >> 1) << 3);
                        const int ci = c0 + n * 8 + 2 * t + (k & 1);
                        if (co < Cout)
                            atomicAdd(dW + (static_cast<size_t>(co) * 27 + tap) * Cin + ci, acc[s][m][n][k]);
                    }
        }
    }

    // ------------------------------------------------------------------ elementwise passes
    __device__ __forceinline__ void unpack8(const uint4& u, float (&f)[8])
    {
        const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 v = __bfloat1622float2(h[k]);
            f[2 * k] = v.x;
            f[2 * k + 1] = v.y;
        }
    }
    __device__ __forceinline__ uint4 pack8(const float (&f)[8])
    {
        uint4 u;
        __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            h[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
        return u;
    }

    // dz = dy * (y > 0), and db[c] += sum dz[., c].  Items are 8 channels (16 B); the
    // grid stride is a multiple of C/8, so each thread keeps one channel group.
    __global__ void reluBackwardKernel(const uint4* __restrict__ dy, const uint4* __restrict__ y,
        uint4* __restrict__ dz, size_t items, int groups, float* __restrict__ db)
    {
        __shared__ float sdb[256];
        for (int i = threadIdx.x; i < 256; i += blockDim.x)
            sdb[i] = 0.0f;
        __syncthreads();
        float s[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
        const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
        const size_t i0 = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
        for (size_t i = i0; i < items; i += stride) {
            float a[8], b[8];
            unpack8(dy[i], a);
            unpack8(y[i], b);
#pragma unroll
            for (int k = 0; k < 8; ++k)
                a[k] = b[k] > 0.0f ? a[k] : 0.0f;
            const uint4 o = pack8(a);
            dz[i] = o;
            float c[8];
            unpack8(o, c); // the bias gradient sums what the other gradients see
#pragma unroll
            for (int k = 0; k < 8; ++k)
                s[k] += c[k];
        }
        const int grp = static_cast<int>(i0 % groups);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            atomicAdd(&sdb[grp * 8 + k], s[k]);
        __syncthreads();
        for (int c = threadIdx.x; c < groups * 8; c += blockDim.x)
            atomicAdd(db + c, sdb[c]);
    }

    // x_{l+1} = mean over the 2x2x2 children (half resolution output)
    __global__ void avgPoolKernel(const uint4* __restrict__ x, uint4* __restrict__ out, int B, int D, int H, int W,
        int groups)
    {
        const int Dh = D >> 1, Hh = H >> 1, Wh = W >> 1;
        const size_t items = static_cast<size_t>(B) * Dh * Hh * Wh * groups;
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < items;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const int g = static_cast<int>(i % groups);
            size_t v = i / groups;
            const int x0 = static_cast<int>(v % Wh) * 2;
            v /= Wh;
            const int y0 = static_cast<int>(v % Hh) * 2;
            v /= Hh;
            const int z0 = static_cast<int>(v % Dh) * 2;
            const size_t b = v / Dh;
            float s[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const size_t src = (((b * D + z0 + (c >> 2)) * H + y0 + ((c >> 1) & 1)) * W + x0 + (c & 1)) * groups + g;
                float f[8];
                unpack8(x[src], f);
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    s[k] += f[k];
            }
#pragma unroll
            for (int k = 0; k < 8; ++k)
                s[k] *= 0.125f;
            out[i] = pack8(s);
        }
    }

    // Gradient of the decoder's concat input, split: du (half resolution, channels
    // [0, cu)) = sum of the 2x2x2 children; de (full resolution, channels [cu, cu+cs))
    // = dcat + dxNext(parent) / 8, the skip path plus the pooled path of the encoder.
    __global__ void splitConcatGradKernel(const uint4* __restrict__ dcat, int gu, int gs,
        const uint4* __restrict__ dxNext, uint4* __restrict__ du, uint4* __restrict__ de, int B, int D, int H, int W)
    {
        const int gc = gu + gs;
        const int Dh = D >> 1, Hh = H >> 1, Wh = W >> 1;
        const size_t nU = du ? static_cast<size_t>(B) * Dh * Hh * Wh * gu : 0;
        const size_t nE = de ? static_cast<size_t>(B) * D * H * W * gs : 0;
        const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < nU + nE; i += stride) {
            if (i < nU) {
                const int g = static_cast<int>(i % gu);
                size_t v = i / gu;
                const int x0 = static_cast<int>(v % Wh) * 2;
                v /= Wh;
                const int y0 = static_cast<int>(v % Hh) * 2;
                v /= Hh;
                const int z0 = static_cast<int>(v % Dh) * 2;
                const size_t b = v / Dh;
                float s[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const size_t src
                        = (((b * D + z0 + (c >> 2)) * H + y0 + ((c >> 1) & 1)) * W + x0 + (c & 1)) * gc + g;
                    float f[8];
                    unpack8(dcat[src], f);
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        s[k] += f[k];
                }
                du[i] = pack8(s);
            } else {
                const size_t j = i - nU;
                const int g = static_cast<int>(j % gs);
                size_t v = j / gs;
                const int x = static_cast<int>(v % W);
                v /= W;
                const int y = static_cast<int>(v % H);
                v /= H;
                const int z = static_cast<int>(v % D);
                const size_t b = v / D;
                float a[8], n[8];
                unpack8(dcat[(((b * D + z) * H + y) * W + x) * gc + gu + g], a);
                unpack8(dxNext[(((b * Dh + (z >> 1)) * Hh + (y >> 1)) * Wh + (x >> 1)) * gs + g], n);
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    a[k] += n[k] * 0.125f;
                de[j] = pack8(a);
            }
        }
    }

    // Head: pred = d . w + b per voxel; in training also the L1 loss and its
    // gradients (dd = g w, dw += g d, db += g with g = sign(pred - target) / N).
    template <int C0>
    __global__ void headKernel(const __nv_bfloat16* __restrict__ d, const float* __restrict__ hw, size_t nvox,
        const float* __restrict__ target, float invN, float* __restrict__ pred, double predScale,
        double* __restrict__ predOut, __nv_bfloat16* __restrict__ dd, float* __restrict__ dhw,
        double* __restrict__ lossSum)
    {
        float w[C0];
#pragma unroll
        for (int c = 0; c < C0; ++c)
            w[c] = hw[c];
        const float b = hw[C0];
        float gw[C0];
#pragma unroll
        for (int c = 0; c < C0; ++c)
            gw[c] = 0.0f;
        float gb = 0.0f, loss = 0.0f;
        for (size_t v = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; v < nvox;
             v += static_cast<size_t>(gridDim.x) * blockDim.x) {
            float x[C0];
            const uint4* src = reinterpret_cast<const uint4*>(d + v * C0);
#pragma unroll
            for (int k = 0; k < C0 / 8; ++k) {
                float f[8];
                unpack8(src[k], f);
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    x[8 * k + j] = f[j];
            }
            float p = b;
#pragma unroll
            for (int c = 0; c < C0; ++c)
                p = fmaf(x[c], w[c], p);
            if (pred)
                pred[v] = p;
            if (predOut)
                predOut[v] = static_cast<double>(p) * predScale;
            if (target) {
                const float diff = p - target[v];
                loss += fabsf(diff);
                const float g = diff > 0.0f ? invN : (diff < 0.0f ? -invN : 0.0f);
                gb += g;
                float o[C0];
#pragma unroll
                for (int c = 0; c < C0; ++c) {
                    gw[c] = fmaf(g, x[c], gw[c]);
                    o[c] = g * w[c];
                }
                uint4* dst = reinterpret_cast<uint4*>(dd + v * C0);
#pragma unroll
                for (int k = 0; k < C0 / 8; ++k) {
                    float f[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        f[j] = o[8 * k + j];
                    dst[k] = pack8(f);
                }
            }
        }
        if (!target)
            return;
        // warp sums, then one atomic per warp
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            gb += __shfl_xor_sync(0xffffffffu, gb, o);
            loss += __shfl_xor_sync(0xffffffffu, loss, o);
#pragma unroll
            for (int c = 0; c < C0; ++c)
                gw[c] += __shfl_xor_sync(0xffffffffu, gw[c], o);
        }
        if ((threadIdx.x & 31) == 0) {
#pragma unroll
            for (int c = 0; c < C0; ++c)
                atomicAdd(dhw + c, gw[c]);
            atomicAdd(dhw + C0, gb);
            atomicAdd(lossSum, static_cast<double>(loss));
        }
    }

    // Adam (Kingma & Ba 2015) on the FP32 master copy; writes the bf16 copy the
    // convolutions read.  c1 = 1 / (1 - beta1^t), c2 = 1 / (1 - beta2^t).
    __global__ void adamKernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
        float* __restrict__ v, __nv_bfloat16* __restrict__ pb, size_t n, float lr, float b1, float b2, float eps,
        float c1, float c2)
    {
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const float gi = g[i];
            const float mi = b1 * m[i] + (1.0f - b1) * gi;
            const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
            m[i] = mi;
            v[i] = vi;
            const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
            p[i] = pi;
            pb[i] = __float2bfloat16_rn(pi);
        }
    }

    __global__ void toBf16Kernel(const float* __restrict__ p, __nv_bfloat16* __restrict__ pb, size_t n)
    {
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x)
            pb[i] = __float2bfloat16_rn(p[i]);
    }

    // dgrad weights: Wt[ci][t][co] = W[co][26 - t][ci]
    __global__ void transposeWeightsKernel(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt,
        int Cout, int Cin)
    {
        const size_t n = static_cast<size_t>(Cout) * 27 * Cin;
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const int co = static_cast<int>(i % Cout);
            const int t = static_cast<int>((i / Cout) % 27);
            const int ci = static_cast<int>(i / (static_cast<size_t>(Cout) * 27));
            wt[i] = w[(static_cast<size_t>(co) * 27 + (26 - t)) * Cin + ci];
        }
    }

    // Network input channels for one volume: [log(1 + d / s), density, one-hot of
    // material 0..5, zeros]; d, density and material come either from arrays or
    // straight from a world (tally energy -> dose, packed voxel words), in which case
    // the bricks holding a non-air voxel are marked too when marks.active is set.
    __global__ void prepareInputKernel(const float* __restrict__ dose, const float* __restrict__ dens,
        const uint8_t* __restrict__ mat, const Tally* __restrict__ tally, const uint32_t* __restrict__ vox,
        double toDose, size_t n, float invScale, uint4* __restrict__ out, const BrickMarks marks)
    {
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            float d, rho;
            int m;
            if (tally) {
                const uint32_t w = vox[i];
                rho = __uint_as_float(w & 0xffffff00u);
                m = static_cast<int>(w & 0xffu);
                // air (material 0) enters with zero dose, as the worker's readout deletes it
                d = rho > 0.0f && m != 0 ? static_cast<float>(tally[i].e * (toDose / rho)) : 0.0f;
                if (marks.active && m != 0) {
                    const uint32_t v = static_cast<uint32_t>(i);
                    const uint32_t row = v / static_cast<uint32_t>(marks.nx);
                    const int x = static_cast<int>(v - row * static_cast<uint32_t>(marks.nx));
                    const int y = static_cast<int>(row % static_cast<uint32_t>(marks.ny));
                    const int z = static_cast<int>(row / static_cast<uint32_t>(marks.ny));
                    marks.active[x / marks.bx + marks.cx * (y / marks.by + marks.cy * (z / marks.bz))] = 1;
                }
            } else {
                d = dose[i];
                rho = dens[i];
                m = mat[i];
            }
            float f[8];
            f[0] = log1pf(fmaxf(d, 0.0f) * invScale);
            f[1] = rho;
#pragma unroll
            for (int k = 0; k < 6; ++k)
                f[2 + k] = m == k ? 1.0f : 0.0f;
            out[2 * i] = pack8(f);
            out[2 * i + 1] = make_uint4(0u, 0u, 0u, 0u);
        }
    }

    // Copy nPatch cubes of edge P from volumes (input 16 channels, target f32) at the
    // given origins into batch tensors.  origins[p] = {volume, z, y, x}.
    __global__ void gatherPatchesKernel(const uint4* const* __restrict__ inputs, const float* const* __restrict__ targets,
        const int* __restrict__ dims, int nVolumes, const int4* __restrict__ origins, int nPatch, int P,
        uint4* __restrict__ xin, float* __restrict__ tgt)
    {
        const size_t per = static_cast<size_t>(P) * P * P;
        const size_t items = per * nPatch * 3; // two 16-byte halves of input + one target per voxel
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < items;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const int part = static_cast<int>(i % 3);
            const size_t v = i / 3;
            const int pt = static_cast<int>(v / per);
            const size_t w = v % per;
            const int x = static_cast<int>(w % P), y = static_cast<int>((w / P) % P), z = static_cast<int>(w / (P * P));
            const int4 o = origins[pt];
            bool ok = o.x >= 0 && o.x < nVolumes;
            int D = 0, H = 0, W = 0;
            if (ok) {
                D = dims[3 * o.x];
                H = dims[3 * o.x + 1];
                W = dims[3 * o.x + 2];
                ok = o.y >= 0 && o.z >= 0 && o.w >= 0 && o.y + z < D && o.z + y < H && o.w + x < W;
            }
            const size_t src = ok ? (static_cast<size_t>(o.y + z) * H + (o.z + y)) * W + (o.w + x) : 0;
            if (part < 2)
                xin[2 * v + part] = ok ? inputs[o.x][2 * src + part] : make_uint4(0u, 0u, 0u, 0u);
            else
                tgt[v] = ok ? targets[o.x][src] : 0.0f;
        }
    }

    // sum and count of the dose over voxels denser than rhoMin (the normalisation scale).
    // The factor toDose / rho is formed in FP32 (relative error ~1e-7, well inside what
    // a normalisation needs): an FP64 division per voxel made this pass FP64-bound.
    __global__ void doseMeanKernel(const Tally* __restrict__ tally, const uint32_t* __restrict__ vox, float toDose,
        size_t n, float rhoMin, double* __restrict__ sum, unsigned long long* __restrict__ count)
    {
        double s = 0.0;
        unsigned long long c = 0;
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const float rho = __uint_as_float(vox[i] & 0xffffff00u);
            if (rho > rhoMin) {
                s += tally[i].e * static_cast<double>(toDose / rho);
                ++c;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
        }
        if ((threadIdx.x & 31) == 0 && c) {
            atomicAdd(sum, s);
            atomicAdd(count, c);
        }
    }

    int grid1d(size_t items)
    {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const size_t blocks = (items + 255) / 256;
        const size_t cap = static_cast<size_t>(sms > 0 ? sms : 1) * 8;
        return static_cast<int>(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
    }
} // namespace

size_t conv3SmemBytes(int nt) { return 2 * static_cast<size_t>(kHaloBytes + 27 * nt * 32); }
size_t wgradSmemBytes(int nt) { return static_cast<size_t>(kHaloBytes) + 512 * nt * 2; }

cudaError_t conv3Configure()
{
    cudaError_t e = cudaFuncSetAttribute(conv3Kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        static_cast<int>(conv3SmemBytes(16)));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(conv3Kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
            static_cast<int>(conv3SmemBytes(32)));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(wgradKernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
            static_cast<int>(wgradSmemBytes(16)));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(wgradKernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
            static_cast<int>(wgradSmemBytes(32)));
    return e;
}

cudaError_t launchConv3(const ConvIn& in, int B, int D, int H, int W, int Cin, const __nv_bfloat16* w,
    const float* bias, int Cout, bool relu, __nv_bfloat16* out, cudaStream_t s)
{
    if (Cin % 16 || Cout % 16 || (in.ca % 16) || (in.b && in.cb % 16) || in.ca + (in.b ? in.cb : 0) != Cin)
        return cudaErrorInvalidValue;
    const int bricks = B * ((D + 7) / 8) * ((H + 7) / 8) * ((W + 7) / 8);
    if (Cout % 32 == 0) {
        conv3Kernel<32><<<dim3(bricks, Cout / 32), 256, conv3SmemBytes(32), s>>>(in, D, H, W, Cin, w, bias, Cout,
            relu ? 1 : 0, out);
    } else {
        conv3Kernel<16><<<dim3(bricks, Cout / 16), 256, conv3SmemBytes(16), s>>>(in, D, H, W, Cin, w, bias, Cout,
            relu ? 1 : 0, out);
    }
    return cudaGetLastError();
}

cudaError_t launchWgrad(const ConvIn& in, const __nv_bfloat16* dz, int B, int D, int H, int W, int Cin, int Cout,
    float* dW, cudaStream_t s)
{
    if (Cin % 16 || Cout % 16)
        return cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int bricks = B * ((D + 7) / 8) * ((H + 7) / 8) * ((W + 7) / 8);
    const int nt = Cout % 32 == 0 ? 32 : 16;
    const int tiles = (Cout / nt) * (Cin / 16);
    int gx = (2 * sms + tiles - 1) / tiles;
    gx = gx < 1 ? 1 : (gx > bricks ? bricks : gx);
    const dim3 grid(gx, Cout / nt, Cin / 16);
    if (nt == 32)
        wgradKernel<32><<<grid, 256, wgradSmemBytes(32), s>>>(in, dz, D, H, W, Cin, Cout, bricks, dW);
    else
        wgradKernel<16><<<grid, 256, wgradSmemBytes(16), s>>>(in, dz, D, H, W, Cin, Cout, bricks, dW);
    return cudaGetLastError();
}

cudaError_t launchReluBackward(const __nv_bfloat16* dy, const __nv_bfloat16* y, __nv_bfloat16* dz, size_t nvox,
    int C, float* db, cudaStream_t s)
{
    if (C % 8 || 256 % (C / 8))
        return cudaErrorInvalidValue;
    const size_t items = nvox * (C / 8);
    reluBackwardKernel<<<grid1d(items), 256, 0, s>>>(reinterpret_cast<const uint4*>(dy),
        reinterpret_cast<const uint4*>(y), reinterpret_cast<uint4*>(dz), items, C / 8, db);
    return cudaGetLastError();
}

cudaError_t launchAvgPool(const __nv_bfloat16* x, __nv_bfloat16* out, int B, int D, int H, int W, int C,
    cudaStream_t s)
{
    const size_t items = static_cast<size_t>(B) * (D / 2) * (H / 2) * (W / 2) * (C / 8);
    avgPoolKernel<<<grid1d(items), 256, 0, s>>>(reinterpret_cast<const uint4*>(x), reinterpret_cast<uint4*>(out), B,
        D, H, W, C / 8);
    return cudaGetLastError();
}

cudaError_t launchSplitConcatGrad(const __nv_bfloat16* dcat, int cu, int cs, const __nv_bfloat16* dxNext,
    __nv_bfloat16* du, __nv_bfloat16* de, int B, int D, int H, int W, cudaStream_t s)
{
    const size_t items = (du ? static_cast<size_t>(B) * (D / 2) * (H / 2) * (W / 2) * (cu / 8) : 0)
        + (de ? static_cast<size_t>(B) * D * H * W * (cs / 8) : 0);
    splitConcatGradKernel<<<grid1d(items), 256, 0, s>>>(reinterpret_cast<const uint4*>(dcat), cu / 8, cs / 8,
        reinterpret_cast<const uint4*>(dxNext), reinterpret_cast<uint4*>(du), reinterpret_cast<uint4*>(de), B, D, H,
        W);
    return cudaGetLastError();
}

cudaError_t launchHead(const __nv_bfloat16* d, int C0, const float* hw, size_t nvox, const float* target,
    float* pred, double predScale, double* predOut, __nv_bfloat16* dd, float* dhw, double* lossSum, cudaStream_t s)
{
    const float invN = nvox ? 1.0f / static_cast<float>(nvox) : 0.0f;
    const int g = grid1d(nvox);
    if (C0 == 16)
        headKernel<16><<<g, 256, 0, s>>>(d, hw, nvox, target, invN, pred, predScale, predOut, dd, dhw, lossSum);
    else if (C0 == 32)
        headKernel<32><<<g, 256, 0, s>>>(d, hw, nvox, target, invN, pred, predScale, predOut, dd, dhw, lossSum);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launchAdam(float* p, const float* g, float* m, float* v, __nv_bfloat16* pb, size_t n, float lr, float b1,
    float b2, float eps, float c1, float c2, cudaStream_t s)
{
    adamKernel<<<grid1d(n), 256, 0, s>>>(p, g, m, v, pb, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t launchToBf16(const float* p, __nv_bfloat16* pb, size_t n, cudaStream_t s)
{
    toBf16Kernel<<<grid1d(n), 256, 0, s>>>(p, pb, n);
    return cudaGetLastError();
}

cudaError_t launchTransposeWeights(const __nv_bfloat16* w, __nv_bfloat16* wt, int Cout, int Cin, cudaStream_t s)
{
    transposeWeightsKernel<<<grid1d(static_cast<size_t>(Cout) * 27 * Cin), 256, 0, s>>>(w, wt, Cout, Cin);
    return cudaGetLastError();
}

cudaError_t launchPrepareInput(const float* dose, const float* dens, const uint8_t* mat, const Tally* tally,
    const uint32_t* vox, double toDose, size_t n, float invScale, __nv_bfloat16* out, cudaStream_t s,
    const BrickMarks* marks)
{
    const BrickMarks none {};
    const BrickMarks& bm = marks ? *marks : none;
    if (bm.active
        && (!tally || n >= (1ull << 32) || bm.nx < 1 || bm.ny < 1 || bm.bx < 1 || bm.by < 1 || bm.bz < 1
            || static_cast<size_t>(bm.nx) * bm.ny == 0 || n % (static_cast<size_t>(bm.nx) * bm.ny) != 0
            || bm.cx < (bm.nx + bm.bx - 1) / bm.bx || bm.cy < (bm.ny + bm.by - 1) / bm.by))
        return cudaErrorInvalidValue;
    prepareInputKernel<<<grid1d(n), 256, 0, s>>>(dose, dens, mat, tally, vox, toDose, n, invScale,
        reinterpret_cast<uint4*>(out), bm);
    return cudaGetLastError();
}

cudaError_t launchGatherPatches(const __nv_bfloat16* const* inputs, const float* const* targets, const int* dims,
    int nVolumes, const int* origins, int nPatch, int P, __nv_bfloat16* xin, float* tgt, cudaStream_t s)
{
    const size_t items = static_cast<size_t>(P) * P * P * nPatch * 3;
    gatherPatchesKernel<<<grid1d(items), 256, 0, s>>>(reinterpret_cast<const uint4* const*>(inputs), targets, dims,
        nVolumes, reinterpret_cast<const int4*>(origins), nPatch, P, reinterpret_cast<uint4*>(xin), tgt);
    return cudaGetLastError();
}

cudaError_t launchDoseMean(const Tally* tally, const uint32_t* vox, double toDose, size_t n, float rhoMin,
    double* sum, unsigned long long* count, cudaStream_t s)
{
    doseMeanKernel<<<grid1d(n), 256, 0, s>>>(tally, vox, static_cast<float>(toDose), n, rhoMin, sum, count);
    return cudaGetLastError();
}

} // namespace nn
} // namespace dxmcg
