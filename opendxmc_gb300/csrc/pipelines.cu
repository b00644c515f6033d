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
    // (on GB300 the two FP64 divisions per voxel would otherwise bound the pass); the
    // table sits in shared memory, and whether a value is such an integer is read from
    // its IEEE-754 bits with integer operations (FP64 runs at a small fraction of the
    // integer rate here).  Any other value is computed.

    // table slot of h when h is an integer in the table's range (+-0 is 0; NaN, the
    // infinities and subnormals are not)
    __device__ __forceinline__ bool lutSlot(double h, int& k)
    {
        const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(h));
        const int e = static_cast<int>((b >> 52) & 0x7ffu) - 1023;
        if (e < 0) {
            if ((b << 1) != 0ull)
                return false;
            k = -kSegLutMin;
            return true;
        }
        if (e > 13) // |h| >= 2^14, beyond every table entry
            return false;
        const unsigned long long mant = (b & 0xfffffffffffffull) | (1ull << 52);
        const int frac = 52 - e;
        if (mant & ((1ull << frac) - 1ull))
            return false;
        const long long mag = static_cast<long long>(mant >> frac);
        const long long v = (b >> 63) ? -mag : mag;
        if (v < kSegLutMin || v >= kSegLutMin + kSegLutSize)
            return false;
        k = static_cast<int>(v - kSegLutMin);
        return true;
    }

    __device__ __forceinline__ void segmentOne(double h, const SegTable& t, const double* lutD, const uint8_t* lutM,
        uint8_t& m, double& d)
    {
        int k;
        if (lutD && lutSlot(h, k)) {
            m = lutM[k];
            d = lutD[k];
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
        const double* __restrict__ gLutD, const uint8_t* __restrict__ gLutM, uint8_t* __restrict__ mat,
        double* __restrict__ dens, int vec)
    {
        __shared__ double sD[kSegLutSize];
        __shared__ uint8_t sM[kSegLutSize];
        if (gLutD) {
            for (int i = threadIdx.x; i < kSegLutSize; i += blockDim.x) {
                sD[i] = __ldg(gLutD + i);
                sM[i] = __ldg(gLutM + i);
            }
            __syncthreads();
        }
        const double* lutD = gLutD ? sD : nullptr;
        const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
        const size_t nq = n / 4;
        size_t q = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
        if (vec) {
            for (; q < nq; q += stride) {
                const double2 a = __ldcs(reinterpret_cast<const double2*>(hu) + 2 * q);
                const double2 b = __ldcs(reinterpret_cast<const double2*>(hu) + 2 * q + 1);
                uchar4 m;
                double2 da, db;
                segmentOne(a.x, t, lutD, sM, m.x, da.x);
                segmentOne(a.y, t, lutD, sM, m.y, da.y);
                segmentOne(b.x, t, lutD, sM, m.z, db.x);
                segmentOne(b.y, t, lutD, sM, m.w, db.y);
                __stcs(reinterpret_cast<uchar4*>(mat) + q, m);
                __stcs(reinterpret_cast<double2*>(dens) + 2 * q, da);
                __stcs(reinterpret_cast<double2*>(dens) + 2 * q + 1, db);
            }
            q = 4 * nq + blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; // the tail
        }
        for (; q < n; q += stride)
            segmentOne(hu[q], t, lutD, sM, mat[q], dens[q]);
    }

    // ---------------------------------------------------------------- organ dose table
    // Every warp takes a contiguous chunk of the volume, 32 consecutive voxels per
    // step, so a lane sees long runs of one label in organ maps.  A lane keeps
    // running sums for its current label and adds them to the block's shared-memory
    // histograms only when the label changes; the block flushes once at the end.
    // FP64 runs at a small fraction of the FP32 rate here, so the per-voxel FP64 work
    // is one add for the density and one fused multiply-add for dose x density (array
    // form) or one add of the tally energy (world form); the constant factors -- voxel
    // volume, and mGy per keV/g -- multiply the block sums.
    struct OrganInputs {
        const uint8_t* organ;
        // array form: dose (any unit) and density per voxel
        const double* dose;
        const double* density;
        // world form: tally and packed voxel words; dose x mass = e * toDose * volume
        const Tally* tally;
        const uint32_t* vox;
        double toDose;
        int airMask; // world form: dose of material-0 voxels counts as 0
        double voxelVolume;
    };

    struct OrganRun {
        unsigned key = 0xffffffffu;
        unsigned count = 0;
        double rho = 0.0, e = 0.0;
    };

    __device__ __forceinline__ void flushRun(OrganRun& r, unsigned* sCnt, double* sRho, double* sE)
    {
        if (r.count) {
            atomicAdd(&sCnt[r.key], r.count);
            atomicAdd(&sRho[r.key], r.rho);
            atomicAdd(&sE[r.key], r.e);
        }
        r.count = 0;
        r.rho = 0.0;
        r.e = 0.0;
    }

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
        const size_t warps = static_cast<size_t>(gridDim.x) * (blockDim.x >> 5);
        const size_t w = static_cast<size_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
        const size_t groups = (n + 31) / 32;
        const size_t g0 = groups * w / warps, g1 = groups * (w + 1) / warps;
        constexpr int kBatch = 4; // 32-voxel steps whose loads are in flight together
        OrganRun run;
        for (size_t g = g0; g < g1; g += kBatch) {
            unsigned o[kBatch];
            double a[kBatch], b[kBatch];
            uint32_t word[kBatch];
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                const size_t i = (g + k) * 32 + lane;
                o[k] = 256u;
                a[k] = b[k] = 0.0;
                word[k] = 0u;
                if (g + k < g1 && i < n) {
                    o[k] = __ldcs(in.organ + i);
                    if (o[k] < static_cast<unsigned>(nOrgans)) {
                        if (WORLD) {
                            word[k] = __ldcs(in.vox + i);
                            a[k] = __ldcs(&in.tally[i].e);
                        } else {
                            a[k] = __ldcs(in.dose + i);
                            b[k] = __ldcs(in.density + i);
                        }
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                if (o[k] >= static_cast<unsigned>(nOrgans))
                    continue;
                if (o[k] != run.key) {
                    flushRun(run, sCnt, sRho, sE);
                    run.key = o[k];
                }
                ++run.count;
                if (WORLD) {
                    const float rho = __uint_as_float(word[k] & 0xffffff00u);
                    run.rho += static_cast<double>(rho);
                    const bool masked = in.airMask && (word[k] & 0xffu) == 0u;
                    if (rho > 0.0f && !masked)
                        run.e += a[k];
                } else {
                    run.rho += b[k];
                    run.e = fma(a[k], b[k], run.e);
                }
            }
        }
        flushRun(run, sCnt, sRho, sE);
        __syncthreads();
        const double eScale = WORLD ? in.toDose * in.voxelVolume : in.voxelVolume;
        for (int i = threadIdx.x; i < nOrgans; i += blockDim.x)
            if (sCnt[i]) {
                atomicAdd(&cnt[i], static_cast<unsigned long long>(sCnt[i]));
                atomicAdd(&sumRho[i], sRho[i]);
                atomicAdd(&sumE[i], sE[i] * eScale);
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
