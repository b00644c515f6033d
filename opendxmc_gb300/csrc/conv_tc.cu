// conv_tc.cu -- tcgen05 (5th-generation tensor core) kernels of the dose denoiser.
// This part has no counterpart in the reference.
//
// ummaProbeKernel is the self-test of the inline-PTX interface in umma.cuh: one CTA
// stages A (128 x 16) and two B tiles (N x 16) in the no-swizzle K-major layout,
// issues three MMAs into two TMEM accumulators -- the first two sharing A through
// the A-operand collector (fill, lastuse), the third accumulating -- and reads the
// accumulators back.  Its buffer is laid out so that every access stays inside the
// 64 KB of shared memory it owns whichever stride of a descriptor is taken along K.
#include <cstdint>

#include <cuda_runtime.h>

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

} // namespace

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
