// aux_kernels.cu -- kernels around the transport: voxel packing, gather-skip cell
// bounds and the two-region Woodcock box at World::build, dose finalisation at
// readout, and the device test hooks that run single pieces of the hot path
// (traversal, history streams, samplers, source) on given inputs.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>

#include "device.cuh"

namespace dxmcg {
namespace {
    using namespace dev;

    // ---------------------------------------------------------------- world build
    __global__ void packKernel(const double* __restrict__ d64, const float* __restrict__ d32,
        const uint8_t* __restrict__ mat, uint32_t* __restrict__ vox, size_t n, int nMats,
        unsigned* __restrict__ rhoMax, unsigned* __restrict__ err)
    {
        __shared__ unsigned smax[256];
        for (int i = threadIdx.x; i < 256; i += blockDim.x)
            smax[i] = 0u;
        __syncthreads();
        unsigned e = 0;
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const float rho = d64 ? static_cast<float>(d64[i]) : d32[i];
            const unsigned m = mat[i];
            if (!(rho >= 0.0f) || !isfinite(rho))
                e |= kErrBadDensity;
            if (m >= static_cast<unsigned>(nMats) && m != DXMCG_TRANSPARENT_MATERIAL)
                e |= kErrBadMaterial;
            const unsigned bits = (rho > 0.0f && isfinite(rho)) ? ((__float_as_uint(rho) + 0x80u) & 0xffffff00u) : 0u;
            vox[i] = bits | m;
            if (bits > smax[m])
                atomicMax(&smax[m], bits);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 256; i += blockDim.x)
            if (smax[i])
                atomicMax(&rhoMax[i], smax[i]);
        if (e)
            atomicOr(err, e);
    }

    // One block per macro cell: the largest rho * ratio[m] over the cell's voxels,
    // times (1 + 2^-20).  Transparent voxels contribute 0.
    __global__ void macroScaleKernel(const uint32_t* __restrict__ vox, int nx, int ny, int nz, int mb, int mcx,
        int mcy, const float* __restrict__ ratio, unsigned* __restrict__ scaleBits)
    {
        const int c = blockIdx.x;
        const int cx = c % mcx, cy = (c / mcx) % mcy, cz = c / (mcx * mcy);
        const int x0 = cx * mb, y0 = cy * mb, z0 = cz * mb;
        const int ex = min(mb, nx - x0), ey = min(mb, ny - y0), ez = min(mb, nz - z0);
        const int n = ex * ey * ez;
        float best = 0.0f;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int ix = x0 + i % ex, iy = y0 + (i / ex) % ey, iz = z0 + i / (ex * ey);
            const uint32_t w = vox[ix + static_cast<size_t>(nx) * (iy + static_cast<size_t>(ny) * iz)];
            const int m = static_cast<int>(w & 0xffu);
            if (m != DXMCG_TRANSPARENT_MATERIAL)
                best = fmaxf(best, __uint_as_float(w & 0xffffff00u) * ratio[m]);
        }
        for (int o = 16; o > 0; o >>= 1)
            best = fmaxf(best, __shfl_xor_sync(kFull, best, o));
        __shared__ float warpBest[32];
        if ((threadIdx.x & 31) == 0)
            warpBest[threadIdx.x >> 5] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
            float b = 0.0f;
            for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w)
                b = fmaxf(b, warpBest[w]);
            scaleBits[c] = __float_as_uint(b * (1.0f + 9.5367431640625e-7f));
        }
    }

    // One block per cell of kCellEdge^3 voxels: the largest rho * ratio[m] of its
    // voxels times (1 + 2^-12), or +inf when one of them is transparent.  The margin
    // covers the FP32 roundings of the interpolated tables on both sides of the
    // Woodcock acceptance test (a few units in 2^-24 each).
    __global__ void cellBoundKernel(const uint32_t* __restrict__ vox, int nx, int ny, int nz, int ncx, int ncy,
        const float* __restrict__ ratio, float* __restrict__ bound)
    {
        const int c = blockIdx.x;
        const int cx = c % ncx, cy = (c / ncx) % ncy, cz = c / (ncx * ncy);
        const int x0 = cx * kCellEdge, y0 = cy * kCellEdge, z0 = cz * kCellEdge;
        const int ex = min(kCellEdge, nx - x0), ey = min(kCellEdge, ny - y0), ez = min(kCellEdge, nz - z0);
        const int n = ex * ey * ez;
        float best = 0.0f;
        bool transparent = false;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int ix = x0 + i % ex, iy = y0 + (i / ex) % ey, iz = z0 + i / (ex * ey);
            const uint32_t w = vox[ix + static_cast<size_t>(nx) * (iy + static_cast<size_t>(ny) * iz)];
            const int m = static_cast<int>(w & 0xffu);
            if (m == DXMCG_TRANSPARENT_MATERIAL)
                transparent = true;
            else
                best = fmaxf(best, __uint_as_float(w & 0xffffff00u) * ratio[m]);
        }
        for (int o = 16; o > 0; o >>= 1)
            best = fmaxf(best, __shfl_xor_sync(kFull, best, o));
        transparent = __any_sync(kFull, transparent);
        __shared__ float warpBest[32];
        __shared__ int warpTransparent[32];
        if ((threadIdx.x & 31) == 0) {
            warpBest[threadIdx.x >> 5] = best;
            warpTransparent[threadIdx.x >> 5] = transparent ? 1 : 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float b = 0.0f;
            int tr = 0;
            for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
                b = fmaxf(b, warpBest[w]);
                tr |= warpTransparent[w];
            }
            bound[c] = tr ? __int_as_float(0x7f800000) : b * (1.0f + 2.44140625e-4f);
        }
    }

    // One warp per (y, z) row of voxels, reading x coalesced; per-lane extremes are
    // reduced over the warp and the block, then six atomics per block.
    // T = uint32_t: packed voxel words (material in the low byte); T = uint8_t: materials
    template <typename T>
    __global__ void materialBoxKernel(const T* __restrict__ vox, int nx, int ny, int nz, int* __restrict__ box)
    {
        int lo[3] = { INT_MAX, INT_MAX, INT_MAX }, hi[3] = { -1, -1, -1 };
        const unsigned lane = threadIdx.x & 31u;
        const long long rows = static_cast<long long>(ny) * nz;
        const long long nWarps = static_cast<long long>(gridDim.x) * (blockDim.x >> 5);
        for (long long r = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; r < rows;
             r += nWarps) {
            const T* row = vox + r * nx;
            int xlo = INT_MAX, xhi = -1;
            for (int x = static_cast<int>(lane); x < nx; x += 32) {
                const uint32_t m = static_cast<uint32_t>(__ldg(row + x)) & 0xffu;
                if (m != 0u && m != DXMCG_TRANSPARENT_MATERIAL) {
                    xlo = min(xlo, x);
                    xhi = max(xhi, x);
                }
            }
            if (xhi >= 0) {
                const int y = static_cast<int>(r % ny), z = static_cast<int>(r / ny);
                lo[0] = min(lo[0], xlo);
                hi[0] = max(hi[0], xhi);
                lo[1] = min(lo[1], y);
                hi[1] = max(hi[1], y);
                lo[2] = min(lo[2], z);
                hi[2] = max(hi[2], z);
            }
        }
        __shared__ int sLo[32][3], sHi[32][3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            for (int o = 16; o > 0; o >>= 1) {
                lo[a] = min(lo[a], __shfl_xor_sync(kFull, lo[a], o));
                hi[a] = max(hi[a], __shfl_xor_sync(kFull, hi[a], o));
            }
            if (lane == 0) {
                sLo[threadIdx.x >> 5][a] = lo[a];
                sHi[threadIdx.x >> 5][a] = hi[a];
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w)
                for (int a = 0; a < 3; ++a) {
                    lo[a] = min(lo[a], sLo[w][a]);
                    hi[a] = max(hi[a], sHi[w][a]);
                }
            if (hi[0] >= 0)
                for (int a = 0; a < 3; ++a) {
                    atomicMin(box + a, lo[a]);
                    atomicMax(box + 3 + a, hi[a]);
                }
        }
    }

    __global__ void finalizeKernel(const Tally* __restrict__ t, const uint32_t* __restrict__ vox, size_t n,
        double toDose, double nh, double* __restrict__ dose, double* __restrict__ var,
        unsigned long long* __restrict__ cnt)
    {
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const Tally r = t[i];
            const float rho = __uint_as_float(vox[i] & 0xffffff00u);
            const double s = rho > 0.0f ? toDose / rho : 0.0;
            if (dose)
                dose[i] = r.e * s;
            if (var) {
                const double v = nh > 0 ? (r.e2 - r.e * r.e / nh) : 0.0;
                var[i] = (v > 0.0 ? v : 0.0) * s * s;
            }
            if (cnt)
                cnt[i] = r.n;
        }
    }

    // ---------------------------------------------------------------- test kernels
    __global__ void siddonKernel(int nRays, const float* __restrict__ o, const float* __restrict__ d, int nx, int ny,
        int nz, float sx, float sy, float sz, int cap, long long* __restrict__ idx, float* __restrict__ len,
        int* __restrict__ cnt)
    {
        const int r = blockIdx.x * blockDim.x + threadIdx.x;
        if (r >= nRays)
            return;
        const int dims[3] = { nx, ny, nz };
        const float sp[3] = { sx, sy, sz };
        Siddon s;
        int c = 0;
        if (s.begin(o + 3 * r, d + 3 * r, dims, sp)) {
            while (!s.done) {
                long long v;
                float l, t0;
                s.next(v, l, t0);
                if (l > 0.0f) {
                    if (c < cap) {
                        idx[static_cast<size_t>(r) * cap + c] = v;
                        len[static_cast<size_t>(r) * cap + c] = l;
                    }
                    ++c;
                }
            }
        }
        cnt[r] = c;
    }

    __global__ void streamKernel(unsigned long long key, unsigned long long h0, int nHist, int nDraws,
        uint32_t* __restrict__ out)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= nHist)
            return;
        Rng r;
        r.init(key, h0 + i);
        for (int k = 0; k < nDraws; ++k)
            out[static_cast<size_t>(i) * nDraws + k] = r.raw();
    }

    __global__ void comptonKernel(int n, const float* __restrict__ E, const DevMaterial* __restrict__ M,
        const float* __restrict__ ctab, int correction, const float* __restrict__ u, int stride,
        float* __restrict__ eo, float* __restrict__ co, int* __restrict__ used)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        InjectedUniforms r { u + static_cast<size_t>(i) * stride, stride, 0 };
        unsigned err = 0;
        float cost;
        int ie;
        float fe;
        gridPos(E[i], ie, fe);
        eo[i] = sampleCompton(E[i], M, ctab, ie, fe, correction, r, cost, err);
        co[i] = cost;
        used[i] = r.used;
    }

    __global__ void rayleighKernel(int n, const float* __restrict__ E, const DevMaterial* __restrict__ M,
        const float* __restrict__ rtab, const float* __restrict__ u, int stride, float* __restrict__ co,
        int* __restrict__ used)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        InjectedUniforms r { u + static_cast<size_t>(i) * stride, stride, 0 };
        int ie;
        float fe;
        gridPos(E[i], ie, fe);
        co[i] = sampleRayleigh(rtab, ie, fe, r);
        used[i] = r.used;
    }

    __global__ void photoKernel(int n, const float* __restrict__ E, const DevMaterial* __restrict__ M,
        const float* __restrict__ u, int stride, float* __restrict__ eo, float* __restrict__ dzo,
        int* __restrict__ used)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        InjectedUniforms r { u + static_cast<size_t>(i) * stride, stride, 0 };
        const float Ef = samplePhotoFluorescence(E[i], M, r);
        float dx = 0.0f, dy = 0.0f, dz = 0.0f;
        if (Ef > 0.0f) {
            const float u1 = r.u();
            isotropicDirection(dx, dy, dz, u1, r.u());
        }
        eo[i] = Ef;
        dzo[i] = dz;
        used[i] = r.used;
    }

    __global__ void sourceKernel(const DevJob J, unsigned long long h0, int n, float* __restrict__ out)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        Rng r;
        r.init(J.key, h0 + i);
        Photon ph;
        sampleSource(J, h0 + i, ph, r);
        float* o = out + 8 * static_cast<size_t>(i);
        o[0] = ph.E;
        o[1] = ph.w;
        o[2] = ph.px;
        o[3] = ph.py;
        o[4] = ph.pz;
        o[5] = ph.dx;
        o[6] = ph.dy;
        o[7] = ph.dz;
    }

    int gridFor(size_t n, int block)
    {
        const size_t g = (n + block - 1) / block;
        return static_cast<int>(g < 1 ? 1 : (g > 65535 * 8 ? 65535 * 8 : g));
    }
} // namespace

cudaError_t launchPack(const double* dens64, const float* dens32, const uint8_t* mat, uint32_t* vox, size_t n,
    int n_mats, unsigned* rho_max_bits, unsigned* err, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = static_cast<int>(std::min<size_t>(gridFor(n, 256), static_cast<size_t>(sms) * 8));
    packKernel<<<grid, 256, 0, s>>>(dens64, dens32, mat, vox, n, n_mats, rho_max_bits, err);
    return cudaGetLastError();
}

cudaError_t launchMacroScale(const uint32_t* vox, int nx, int ny, int nz, int mb, int mcx, int mcy,
    const float* ratio, unsigned* scaleBits, cudaStream_t s)
{
    const int mcz = (nz + mb - 1) / mb;
    macroScaleKernel<<<mcx * mcy * mcz, 256, 0, s>>>(vox, nx, ny, nz, mb, mcx, mcy, ratio, scaleBits);
    return cudaGetLastError();
}

cudaError_t launchCellBound(const uint32_t* vox, int nx, int ny, int nz, int ncx, int ncy, int ncz, const float* ratio,
    float* bound, cudaStream_t s)
{
    cellBoundKernel<<<ncx * ncy * ncz, 128, 0, s>>>(vox, nx, ny, nz, ncx, ncy, ratio, bound);
    return cudaGetLastError();
}

static int materialBoxBlocks(int ny, int nz)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long rows = static_cast<long long>(ny) * nz;
    return static_cast<int>(std::min<long long>((rows + 7) / 8, 4LL * (sms > 0 ? sms : 1)));
}

cudaError_t launchMaterialBox(const uint32_t* vox, int nx, int ny, int nz, int* box, cudaStream_t s)
{
    materialBoxKernel<uint32_t><<<materialBoxBlocks(ny, nz), 256, 0, s>>>(vox, nx, ny, nz, box);
    return cudaGetLastError();
}

cudaError_t launchMaterialBox(const uint8_t* mat, int nx, int ny, int nz, int* box, cudaStream_t s)
{
    materialBoxKernel<uint8_t><<<materialBoxBlocks(ny, nz), 256, 0, s>>>(mat, nx, ny, nz, box);
    return cudaGetLastError();
}

cudaError_t launchFinalize(const Tally* tally, const uint32_t* vox, size_t n, double energy_to_dose,
    double n_histories, double* dose, double* var, unsigned long long* count, cudaStream_t s)
{
    finalizeKernel<<<gridFor(n, 256), 256, 0, s>>>(tally, vox, n, energy_to_dose, n_histories, dose, var, count);
    return cudaGetLastError();
}

cudaError_t launchSiddon(int n_rays, const float* o, const float* d, int nx, int ny, int nz, float sx, float sy,
    float sz, int cap, long long* idx, float* len, int* cnt, cudaStream_t s)
{
    siddonKernel<<<(n_rays + 127) / 128, 128, 0, s>>>(n_rays, o, d, nx, ny, nz, sx, sy, sz, cap, idx, len, cnt);
    return cudaGetLastError();
}

cudaError_t launchHistoryStream(unsigned long long key, unsigned long long h0, int n_hist, int n_draws,
    uint32_t* out, cudaStream_t s)
{
    streamKernel<<<(n_hist + 127) / 128, 128, 0, s>>>(key, h0, n_hist, n_draws, out);
    return cudaGetLastError();
}

cudaError_t launchSampleCompton(int n, const float* E, const DevMaterial* m, const float* ctab, int correction,
    const float* u, int stride, float* e_out, float* cos_out, int* used, cudaStream_t s)
{
    comptonKernel<<<(n + 127) / 128, 128, 0, s>>>(n, E, m, ctab, correction, u, stride, e_out, cos_out, used);
    return cudaGetLastError();
}

cudaError_t launchSamplePhoto(int n, const float* E, const DevMaterial* m, const float* u, int stride, float* e_out,
    float* dz_out, int* used, cudaStream_t s)
{
    photoKernel<<<(n + 127) / 128, 128, 0, s>>>(n, E, m, u, stride, e_out, dz_out, used);
    return cudaGetLastError();
}

cudaError_t launchSampleRayleigh(int n, const float* E, const DevMaterial* m, const float* rtab, const float* u,
    int stride, float* cos_out, int* used, cudaStream_t s)
{
    rayleighKernel<<<(n + 127) / 128, 128, 0, s>>>(n, E, m, rtab, u, stride, cos_out, used);
    return cudaGetLastError();
}

cudaError_t launchSampleSource(const DevJob& job, unsigned long long h0, int n, float* out8, cudaStream_t s)
{
    sourceKernel<<<(n + 127) / 128, 128, 0, s>>>(job, h0, n, out8);
    return cudaGetLastError();
}

} // namespace dxmcg
