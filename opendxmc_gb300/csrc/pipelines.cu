// pipelines.cu -- the per-voxel passes on either side of the transport:
//
//  * CT segmentation (ctsegmentationpipeline.cpp:117-169): HU -> material index by
//    the midpoints between the materials' mean CT numbers, and HU -> density by the
//    water/air calibration line divided by the material's mass attenuation;
//  * organ dose table (dosetablepipeline.cpp:55-85): per organ label the voxel
//    count, sum of density and sum of dose x voxel mass, one pass over the arrays;
//  * dose post-processing at readout (simulationpipeline.cpp:173-231): air mask,
//    the mGy -> uGy switch when the maximum dose is below 1, variance x 1e6 with it.
//
// All three are streaming passes: one read of each input element and one write of
// each output element, so HBM bandwidth bounds them.  FP64 throughout, and the
// per-voxel arithmetic is written with explicitly rounded operations in the
// reference's order, so that a plain FP64 restatement reproduces it bit for bit.
#include <cstdint>

#include "device.cuh"

namespace dxmcg {
namespace {
    using namespace dev;

    // ---------------------------------------------------------------- segmentation
    // Integer CT numbers in [kSegLutMin, kSegLutMin + kSegLutSize) read their result
    // from a table filled once per segmentation table with the same FP64 operations
    // (on GB300 the two FP64 divisions per voxel would otherwise bound the pass);
    // any other value is computed here.
    __device__ __forceinline__ void segmentOne(double h, const SegTable& t, const double* __restrict__ lutD,
        const uint8_t* __restrict__ lutM, uint8_t& m, double& d)
    {
        if (lutD && h == rint(h) && h >= static_cast<double>(kSegLutMin)
            && h < static_cast<double>(kSegLutMin + kSegLutSize)) {
            const int k = static_cast<int>(h) - kSegLutMin;
            m = __ldg(lutM + k);
            d = __ldg(lutD + k);
            return;
        }
        int i = 0;
        while (i < t.nSep && !(h < t.sep[i]))
            ++i;
        m = static_cast<uint8_t>(i);
        // (((w_att w_dens - a_att a_dens) hu / 1000) + w_att w_dens) / m_att, then max(., 0)
        const double v = __ddiv_rn(__dadd_rn(__ddiv_rn(__dmul_rn(t.slope, h), 1000.0), t.offset), t.att[i]);
        d = v < 0.0 ? 0.0 : v;
    }

    // Four voxels per thread and iteration: 32 B of HU in, 4 B of material and 32 B of
    // density out with 16-byte / 4-byte vector accesses (the host checks alignment).
    __global__ void segmentKernel(const double* __restrict__ hu, size_t n, const SegTable t,
        const double* __restrict__ lutD, const uint8_t* __restrict__ lutM, uint8_t* __restrict__ mat,
        double* __restrict__ dens, int vec)
    {
        const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
        const size_t nq = n / 4;
        size_t q = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
        if (vec) {
            for (; q < nq; q += stride) {
                const double2 a = reinterpret_cast<const double2*>(hu)[2 * q];
                const double2 b = reinterpret_cast<const double2*>(hu)[2 * q + 1];
                uchar4 m;
                double2 da, db;
                segmentOne(a.x, t, lutD, lutM, m.x, da.x);
                segmentOne(a.y, t, lutD, lutM, m.y, da.y);
                segmentOne(b.x, t, lutD, lutM, m.z, db.x);
                segmentOne(b.y, t, lutD, lutM, m.w, db.y);
                reinterpret_cast<uchar4*>(mat)[q] = m;
                reinterpret_cast<double2*>(dens)[2 * q] = da;
                reinterpret_cast<double2*>(dens)[2 * q + 1] = db;
            }
            q = 4 * nq + blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; // the tail
        }
        for (; q < n; q += stride)
            segmentOne(hu[q], t, lutD, lutM, mat[q], dens[q]);
    }

    // ---------------------------------------------------------------- organ dose table
    // Per-block histograms over the 256 labels in shared memory, flushed once per
    // block.  Lanes that share a label are combined first (__match_any_sync); a
    // warp whose 32 voxels carry one label -- the common case in organ maps --
    // reduces by shuffles and touches shared memory once.
    struct OrganInputs {
        const uint8_t* organ;
        // array form: dose (any unit) and density per voxel
        const double* dose;
        const double* density;
        // world form: tally and packed voxel words; dose = e * toDose / rho
        const Tally* tally;
        const uint32_t* vox;
        double toDose;
        int airMask; // world form: dose of material-0 voxels counts as 0
        double voxelVolume;
    };

    template <bool WORLD>
    __global__ void organKernel(const OrganInputs in, size_t n, int nOrgans, unsigned long long* __restrict__ cnt,
        double* __restrict__ sumRho, double* __restrict__ sumE)
    {
        __shared__ unsigned sCnt[256];
        __shared__ double sRho[256], sE[256];
        for (int i = threadIdx.x; i < 256; i += blockDim.x) {
            sCnt[i] = 0u;
            sRho[i] = 0.0;
            sE[i] = 0.0;
        }
        __syncthreads();
        const unsigned lane = threadIdx.x & 31u;
        const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
        // the loop bound is uniform per warp so that every lane reaches the warp votes
        for (size_t base = blockIdx.x * static_cast<size_t>(blockDim.x) + (threadIdx.x & ~31u); base < n;
             base += stride) {
            const size_t i = base + lane;
            unsigned key = 256u;
            double rho = 0.0, e = 0.0;
            if (i < n) {
                const unsigned o = in.organ[i];
                if (o < static_cast<unsigned>(nOrgans)) {
                    key = o;
                    if (WORLD) {
                        const uint32_t w = in.vox[i];
                        rho = static_cast<double>(__uint_as_float(w & 0xffffff00u));
                        const bool masked = in.airMask && (w & 0xffu) == 0u;
                        const double d = (rho > 0.0 && !masked) ? in.tally[i].e * (in.toDose / rho) : 0.0;
                        e = d * (in.voxelVolume * rho);
                    } else {
                        rho = in.density[i];
                        e = in.dose[i] * (in.voxelVolume * rho);
                    }
                }
            }
            const unsigned peers = __match_any_sync(kFull, key);
            if (peers == kFull) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    rho += __shfl_xor_sync(kFull, rho, o);
                    e += __shfl_xor_sync(kFull, e, o);
                }
                if (lane == 0 && key < 256u) {
                    atomicAdd(&sCnt[key], 32u);
                    atomicAdd(&sRho[key], rho);
                    atomicAdd(&sE[key], e);
                }
            } else if (key < 256u) {
                if (lane == static_cast<unsigned>(__ffs(peers) - 1))
                    atomicAdd(&sCnt[key], static_cast<unsigned>(__popc(peers)));
                atomicAdd(&sRho[key], rho);
                atomicAdd(&sE[key], e);
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nOrgans; i += blockDim.x)
            if (sCnt[i]) {
                atomicAdd(&cnt[i], static_cast<unsigned long long>(sCnt[i]));
                atomicAdd(&sumRho[i], sRho[i]);
                atomicAdd(&sumE[i], sE[i]);
            }
    }

    // ---------------------------------------------------------------- dose post-processing
    __device__ __forceinline__ double voxelDose(const Tally& r, uint32_t w, double toDose, int airMask)
    {
        const float rho = __uint_as_float(w & 0xffffff00u);
        if (airMask && (w & 0xffu) == 0u)
            return 0.0;
        return rho > 0.0f ? r.e * (toDose / rho) : 0.0;
    }

    // maximum dose (non-negative doubles order like their bit patterns)
    __global__ void doseMaxKernel(const Tally* __restrict__ t, const uint32_t* __restrict__ vox, size_t n,
        double toDose, int airMask, unsigned long long* __restrict__ maxBits)
    {
        double m = 0.0;
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x)
            m = fmax(m, voxelDose(t[i], vox[i], toDose, airMask));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            m = fmax(m, __shfl_xor_sync(kFull, m, o));
        if ((threadIdx.x & 31u) == 0u && m > 0.0)
            atomicMax(maxBits, static_cast<unsigned long long>(__double_as_longlong(m)));
    }

    __global__ void postprocessKernel(const Tally* __restrict__ t, const uint32_t* __restrict__ vox, size_t n,
        double toDose, double nh, int airMask, const unsigned long long* __restrict__ maxBits,
        double* __restrict__ dose, double* __restrict__ var, double* __restrict__ count, int* __restrict__ micro)
    {
        const bool uGy = __longlong_as_double(static_cast<long long>(*maxBits)) < 1.0;
        if (micro && blockIdx.x == 0 && threadIdx.x == 0)
            *micro = uGy ? 1 : 0;
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const Tally r = t[i];
            const uint32_t w = vox[i];
            const bool masked = airMask && (w & 0xffu) == 0u;
            const float rho = __uint_as_float(w & 0xffffff00u);
            const double s = rho > 0.0f ? toDose / rho : 0.0;
            if (dose) {
                const double d = masked ? 0.0 : r.e * s;
                dose[i] = uGy ? d * 1e3 : d;
            }
            if (var) {
                const double v0 = nh > 0 ? (r.e2 - r.e * r.e / nh) : 0.0;
                const double v = masked ? 0.0 : (v0 > 0.0 ? v0 : 0.0) * s * s;
                var[i] = uGy ? v * 1e6 : v;
            }
            if (count)
                count[i] = masked ? 0.0 : static_cast<double>(r.n);
        }
    }

    int streamingGrid(size_t work)
    {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const size_t blocks = (work + 255) / 256;
        const size_t cap = static_cast<size_t>(sms > 0 ? sms : 1) * 8; // 8 blocks of 256 per SM
        return static_cast<int>(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
    }
} // namespace

cudaError_t launchSegment(const double* hu, size_t n, const SegTable& t, const double* lutD, const uint8_t* lutM,
    uint8_t* mat, double* dens, cudaStream_t s)
{
    const bool vec = (reinterpret_cast<uintptr_t>(hu) % 16 == 0) && (reinterpret_cast<uintptr_t>(dens) % 16 == 0)
        && (reinterpret_cast<uintptr_t>(mat) % 4 == 0);
    segmentKernel<<<streamingGrid(vec ? n / 4 : n), 256, 0, s>>>(hu, n, t, lutD, lutM, mat, dens, vec ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launchOrganTable(const uint8_t* organ, const double* dose, const double* density, size_t n,
    double voxel_volume, int n_organs, unsigned long long* cnt, double* sum_rho, double* sum_e, cudaStream_t s)
{
    OrganInputs in {};
    in.organ = organ;
    in.dose = dose;
    in.density = density;
    in.voxelVolume = voxel_volume;
    organKernel<false><<<streamingGrid(n), 256, 0, s>>>(in, n, n_organs, cnt, sum_rho, sum_e);
    return cudaGetLastError();
}

cudaError_t launchWorldOrganTable(const uint8_t* organ, const Tally* tally, const uint32_t* vox, size_t n,
    double energy_to_dose, int air_mask, double voxel_volume, int n_organs, unsigned long long* cnt,
    double* sum_rho, double* sum_e, cudaStream_t s)
{
    OrganInputs in {};
    in.organ = organ;
    in.tally = tally;
    in.vox = vox;
    in.toDose = energy_to_dose;
    in.airMask = air_mask;
    in.voxelVolume = voxel_volume;
    organKernel<true><<<streamingGrid(n), 256, 0, s>>>(in, n, n_organs, cnt, sum_rho, sum_e);
    return cudaGetLastError();
}

cudaError_t launchDosePostprocess(const Tally* tally, const uint32_t* vox, size_t n, double energy_to_dose,
    double n_histories, int air_mask, unsigned long long* max_bits, double* dose, double* var, double* count,
    int* micro, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(max_bits, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess)
        return e;
    const int g = streamingGrid(n);
    doseMaxKernel<<<g, 256, 0, s>>>(tally, vox, n, energy_to_dose, air_mask, max_bits);
    postprocessKernel<<<g, 256, 0, s>>>(tally, vox, n, energy_to_dose, n_histories, air_mask, max_bits, dose, var,
        count, micro);
    return cudaGetLastError();
}

} // namespace dxmcg
