// noalloc.cu -- the transport entry point that allocates no device memory.
//
// Who needs it: callers that may not call cudaMalloc (or any other device
// allocator) while they run a simulation -- an application whose GPU memory is
// handed out only by its own pool allocator, a plugin host that gives each
// plugin a fixed device-memory budget up front, a service that must not allocate
// between its set-up phase and its runs.  They own every input and output array
// and pass device pointers; everything else this path needs -- the work-queue head
// and run statistics, the validation flags and per-material maximum densities,
// the attenuation tables and majorants, the Compton angle and Rayleigh share tables,
// the two-region box, the exposure list, the spectra and the bowtie profiles -- lives
// in one file-scope __device__ array of kScratchBytes = 12 MiB.  Every GPU that loads
// the library holds that array until the process exits.
//
// The host finds the array's device address with cudaGetSymbolAddress, once per
// device, with that device current, on the first call made on that device.  Every
// call reads its validation flags back and synchronises its stream partway, and
// again at the end, so no call can be captured into a CUDA graph: a call on a
// capturing stream is refused before it queues any work.  All calls share the
// array and it keeps the last call's contents: each call clears the counters it
// needs to start at zero, and calls that overlap on the GPU (on different streams
// or threads) race on it, so issue them one after another.
//
// Calibration: DX/CBCT beams (dose-area product) and pencil beams (air kerma) are
// normalised analytically; CT beams with a CTDI target are refused, because their
// calibration simulates a CTDI phantom world, which needs device allocations.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dxmcg.h"
#include "engine.hpp"
#include "jobs.hpp"

namespace dxmcg {
namespace {

    constexpr size_t kScratchBytes = 12u * 1024u * 1024u;
    constexpr int kMaxMaterials = 16;
    constexpr int kMaxExposures = 4096;
    constexpr int kMaxDevices = 64;

    static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

    constexpr size_t alignUp(size_t x) { return (x + 255u) & ~static_cast<size_t>(255u); }

    // byte offsets of the pieces inside g_scratch
    constexpr size_t kOffCounters = 0;
    constexpr size_t kOffFlags = alignUp(kOffCounters + sizeof(DevCounters)); // 256 rho-max words + error word
    constexpr size_t kOffSpec = alignUp(kOffFlags + 257 * sizeof(unsigned));
    constexpr size_t kOffBowtie = alignUp(kOffSpec + 2 * sizeof(DevSpectrum));
    constexpr size_t kOffMats = alignUp(kOffBowtie + sizeof(DevBowtie));
    constexpr size_t kOffMaj = alignUp(kOffMats + kMaxMaterials * sizeof(DevMaterial));
    constexpr size_t kOffTot = alignUp(kOffMaj + kTableNE * sizeof(float));
    constexpr size_t kOffXs = alignUp(kOffTot + kMaxMaterials * kTableNE * sizeof(float));
    constexpr size_t kOffExps = alignUp(kOffXs + kMaxMaterials * kTableNE * sizeof(float4));
    constexpr size_t kOffCTab = alignUp(kOffExps + kMaxExposures * sizeof(DevExposure));
    constexpr size_t kOffRTab = alignUp(kOffCTab + kMaxMaterials * kTableNE * kCTabK * sizeof(float));
    constexpr size_t kOffBox = alignUp(kOffRTab + kMaxMaterials * kTableNE * kCTabK * sizeof(float)); // 6 ints
    constexpr size_t kOffMajOut = alignUp(kOffBox + 6 * sizeof(int));
    constexpr size_t kUsed = kOffMajOut + kTableNE * sizeof(float);
    static_assert(kUsed <= kScratchBytes, "scratch layout exceeds the static array");
    static_assert(sizeof(dxmcg_tally_record) == sizeof(Tally), "tally record layout");

    std::mutex g_setupMutex;
    unsigned char* g_address[kMaxDevices] = {};

    int fail(int code, const std::string& msg) { return reportError(code, msg); }

    // Device address of g_scratch on the current device (set up once per device).
    int scratchAddress(unsigned char** out)
    {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess)
            return fail(DXMCG_ERR_NO_DEVICE, std::string("transport_run_noalloc: ") + cudaGetErrorString(e));
        if (dev < 0 || dev >= kMaxDevices)
            return fail(DXMCG_ERR_CAPACITY, "transport_run_noalloc: device ordinal beyond 63");
        std::lock_guard<std::mutex> lock(g_setupMutex);
        if (!g_address[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_scratch);
            if (e != cudaSuccess || !p)
                return fail(DXMCG_ERR_CUDA,
                    std::string("transport_run_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
            g_address[dev] = static_cast<unsigned char*>(p);
        }
        *out = g_address[dev];
        return DXMCG_OK;
    }

    // Per-material maximum density and input validation over the caller's arrays.
    __global__ void rhoMaxKernel(const float* __restrict__ dens, const uint8_t* __restrict__ mat, size_t n, int nMats,
        unsigned* __restrict__ rhoMax, unsigned* __restrict__ err)
    {
        __shared__ unsigned smax[256];
        for (int i = threadIdx.x; i < 256; i += blockDim.x)
            smax[i] = 0u;
        __syncthreads();
        unsigned e = 0;
        for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const float rho = dens[i];
            const unsigned m = mat[i];
            if (!(rho >= 0.0f) || !isfinite(rho))
                e |= kErrBadDensity;
            if (m >= static_cast<unsigned>(nMats) && m != DXMCG_TRANSPARENT_MATERIAL)
                e |= kErrBadMaterial;
            const unsigned bits = (rho > 0.0f && isfinite(rho)) ? __float_as_uint(rho) : 0u;
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

#define NOALLOC_CUDA(call)                                                                             \
    do {                                                                                               \
        const cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                         \
            return fail(DXMCG_ERR_CUDA, std::string("transport_run_noalloc: ") + #call + ": "          \
                    + cudaGetErrorString(e_));                                                         \
    } while (0)

} // namespace
} // namespace dxmcg

using namespace dxmcg;

extern "C" DXMCG_API int dxmcg_transport_run_noalloc(const int32_t dims[3], const double spacing_cm[3],
    const float* device_density, const uint8_t* device_material, const dxmcg_material* materials, int n_materials,
    int correction, const dxmcg_beam* beam, const dxmcg_run_options* opts, dxmcg_tally_record* device_tally,
    void* cuda_stream, dxmcg_stats* stats)
{
    if (!dims || !spacing_cm || !device_density || !device_material || !materials || !beam || !device_tally)
        return fail(DXMCG_ERR_ARGUMENT, "transport_run_noalloc: null argument");
    if ((reinterpret_cast<uintptr_t>(device_tally) & 31u) != 0 || (reinterpret_cast<uintptr_t>(device_density) & 3u) != 0)
        return fail(DXMCG_ERR_ARGUMENT, "transport_run_noalloc: tally must be 32-byte and density 4-byte aligned");
    uint64_t N = 1;
    for (int a = 0; a < 3; ++a) {
        if (dims[a] < 1 || !(spacing_cm[a] > 0))
            return fail(DXMCG_ERR_ARGUMENT, "transport_run_noalloc: dimensions and spacing must be positive");
        N *= static_cast<uint64_t>(dims[a]);
    }
    if (N >= (1ull << 32))
        return fail(DXMCG_ERR_ARGUMENT, "transport_run_noalloc: more than 2^32-1 voxels");
    if (n_materials < 1 || n_materials > kMaxMaterials)
        return fail(DXMCG_ERR_CAPACITY, "transport_run_noalloc: 1 to 16 materials (the scratch array holds 16)");
    for (int m = 0; m < n_materials; ++m)
        if (!validComposition(materials[m]))
            return fail(DXMCG_ERR_ARGUMENT, "transport_run_noalloc: invalid material composition");
    if (correction < 0 || correction > 2)
        return fail(DXMCG_ERR_ARGUMENT, "transport_run_noalloc: correction must be 0, 1 or 2");
    dxmcg_run_options o {};
    o.seed = 1;
    if (opts)
        o = *opts;
    if (o.tracking != DXMCG_TRACK_WOODCOCK && o.tracking != DXMCG_TRACK_SIDDON)
        return fail(DXMCG_ERR_ARGUMENT, "transport_run_noalloc: Woodcock or Siddon tracking only");

    // host-side preparation; sizes are checked against the scratch capacity first
    HostJob hj;
    std::string err;
    int rc = buildHostJob(*beam, dims, spacing_cm, hj, err);
    if (rc != DXMCG_OK)
        return fail(rc, "transport_run_noalloc: " + err);
    if (hj.exposures.size() > static_cast<size_t>(kMaxExposures))
        return fail(DXMCG_ERR_CAPACITY, "transport_run_noalloc: more than 4096 exposures (" +
                std::to_string(hj.exposures.size()) + ") do not fit the scratch array");
    double calibration = 1.0;
    rc = calibrationFactor(*beam, correction, o, hj.nHist, false, calibration, err);
    if (rc != DXMCG_OK)
        return fail(rc, "transport_run_noalloc: " + err);
    if (calibration != 1.0)
        for (auto& e : hj.exposures)
            e.weight = static_cast<float>(e.weight * calibration);

    unsigned char* base = nullptr;
    rc = scratchAddress(&base);
    if (rc != DXMCG_OK)
        return rc;
    const cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    const cudaError_t qe = cudaStreamIsCapturing(s, &capture);
    if (qe != cudaSuccess || capture != cudaStreamCaptureStatusNone) {
        if (qe != cudaSuccess)
            (void)cudaGetLastError();
        return fail(DXMCG_ERR_ARGUMENT,
            "transport_run_noalloc: the stream is being captured; this call synchronises its stream and "
            "cannot be captured into a CUDA graph");
    }
    auto* counters = reinterpret_cast<DevCounters*>(base + kOffCounters);
    auto* flags = reinterpret_cast<unsigned*>(base + kOffFlags);

    // 1. maximum density per material and validation of the caller's arrays; the
    //    two-region box of the materials
    auto* box = reinterpret_cast<int*>(base + kOffBox);
    const int boxInit[6] = { INT_MAX, INT_MAX, INT_MAX, -1, -1, -1 };
    NOALLOC_CUDA(cudaMemsetAsync(flags, 0, 257 * sizeof(unsigned), s));
    NOALLOC_CUDA(cudaMemcpyAsync(box, boxInit, sizeof(boxInit), cudaMemcpyHostToDevice, s));
    int dev = 0, sms = 0;
    NOALLOC_CUDA(cudaGetDevice(&dev));
    NOALLOC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = static_cast<int>(std::min<uint64_t>((N + 255) / 256, static_cast<uint64_t>(sms) * 8));
    rhoMaxKernel<<<grid, 256, 0, s>>>(device_density, device_material, static_cast<size_t>(N), n_materials, flags,
        flags + 256);
    NOALLOC_CUDA(cudaGetLastError());
    const bool woodcock = o.tracking == DXMCG_TRACK_WOODCOCK && o.two_region >= 0;
    if (woodcock)
        NOALLOC_CUDA(launchMaterialBox(device_material, dims[0], dims[1], dims[2], box, s));
    unsigned host[257];
    int hostBox[6];
    NOALLOC_CUDA(cudaMemcpyAsync(host, flags, sizeof(host), cudaMemcpyDeviceToHost, s));
    NOALLOC_CUDA(cudaMemcpyAsync(hostBox, box, sizeof(hostBox), cudaMemcpyDeviceToHost, s));
    NOALLOC_CUDA(cudaStreamSynchronize(s));
    if (host[256] & kErrBadMaterial)
        return fail(DXMCG_ERR_ARGUMENT, "transport_run_noalloc: a voxel's material index is >= the number of materials");
    if (host[256] & kErrBadDensity)
        return fail(DXMCG_ERR_ARGUMENT, "transport_run_noalloc: negative or non-finite density");

    // 2. tables, majorant, exposures, spectra, bowtie into the scratch array
    double rhoMax[kMaxMaterials];
    for (int m = 0; m < n_materials; ++m) {
        float f;
        std::memcpy(&f, &host[m], 4);
        rhoMax[m] = f;
    }
    std::vector<float> tot(static_cast<size_t>(n_materials) * kTableNE);
    std::vector<float4> xs(static_cast<size_t>(n_materials) * kTableNE);
    std::vector<float> maj(kTableNE);
    std::vector<DevMaterial> dm(n_materials);
    buildDeviceTables(materials, n_materials, correction, rhoMax, tot.data(), xs.data(), maj.data(), dm.data());
    NOALLOC_CUDA(cudaMemcpyAsync(base + kOffTot, tot.data(), tot.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    NOALLOC_CUDA(cudaMemcpyAsync(base + kOffXs, xs.data(), xs.size() * sizeof(float4), cudaMemcpyHostToDevice, s));
    std::vector<float> ctab(static_cast<size_t>(n_materials) * kTableNE * kCTabK);
    buildComptonAngleTables(materials, n_materials, correction, ctab.data());
    NOALLOC_CUDA(cudaMemcpyAsync(base + kOffCTab, ctab.data(), ctab.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    std::vector<float> rtab(static_cast<size_t>(n_materials) * kTableNE * kCTabK);
    buildRayleighAngleTables(materials, n_materials, rtab.data());
    NOALLOC_CUDA(cudaMemcpyAsync(base + kOffRTab, rtab.data(), rtab.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    NOALLOC_CUDA(cudaMemcpyAsync(base + kOffMaj, maj.data(), maj.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    const bool twoRegion = woodcock && twoRegionBox(hostBox, dims) && twoRegionFor(o, boxFraction(hostBox, dims));
    std::vector<float> majOut(kTableNE);
    if (twoRegion) {
        buildBackgroundMajorant(tot.data(), rhoMax[0], majOut.data());
        NOALLOC_CUDA(cudaMemcpyAsync(base + kOffMajOut, majOut.data(), majOut.size() * sizeof(float),
            cudaMemcpyHostToDevice, s));
    }
    NOALLOC_CUDA(cudaMemcpyAsync(base + kOffMats, dm.data(), dm.size() * sizeof(DevMaterial), cudaMemcpyHostToDevice, s));
    NOALLOC_CUDA(cudaMemcpyAsync(base + kOffExps, hj.exposures.data(), hj.exposures.size() * sizeof(DevExposure),
        cudaMemcpyHostToDevice, s));
    NOALLOC_CUDA(cudaMemcpyAsync(base + kOffSpec, hj.spec, 2 * sizeof(DevSpectrum), cudaMemcpyHostToDevice, s));
    if (hj.hasBowtie)
        NOALLOC_CUDA(cudaMemcpyAsync(base + kOffBowtie, &hj.bowtie, sizeof(DevBowtie), cudaMemcpyHostToDevice, s));

    // 3. counters start at zero; the queue head at the first history of the range
    const uint64_t h0 = std::min<uint64_t>(o.hist_begin, hj.nHist);
    const uint64_t h1 = o.hist_end == 0 ? hj.nHist : std::min<uint64_t>(o.hist_end, hj.nHist);
    DevCounters zero {};
    zero.next = h0;
    NOALLOC_CUDA(cudaMemcpyAsync(counters, &zero, sizeof(zero), cudaMemcpyHostToDevice, s));

    DevJob J {};
    fillJobFields(J, *beam, o, dims, spacing_cm, correction, n_materials, static_cast<int>(hj.exposures.size()));
    J.vox = nullptr;
    J.dens = device_density;
    J.mat = device_material;
    J.tot = reinterpret_cast<const float*>(base + kOffTot);
    J.xs = reinterpret_cast<const float4*>(base + kOffXs);
    J.ctab = reinterpret_cast<const float*>(base + kOffCTab);
    J.rtab = reinterpret_cast<const float*>(base + kOffRTab);
    J.maj = reinterpret_cast<const float*>(base + kOffMaj);
    J.mats = reinterpret_cast<const DevMaterial*>(base + kOffMats);
    J.tally = reinterpret_cast<Tally*>(device_tally);
    J.exps = reinterpret_cast<const DevExposure*>(base + kOffExps);
    J.spec = reinterpret_cast<const DevSpectrum*>(base + kOffSpec);
    J.bowtie = hj.hasBowtie ? reinterpret_cast<const DevBowtie*>(base + kOffBowtie) : nullptr;
    if (twoRegion)
        setTwoRegion(J, hostBox, spacing_cm, reinterpret_cast<const float*>(base + kOffMajOut));

    LaunchShape shape;
    shape.block = o.block_size > 0 ? std::max(32, std::min(256, o.block_size / 32 * 32)) : 256;
    const int resident = transportMaxBlocksPerSMUnpacked(shape.block, kernelTracking(J));
    shape.grid = std::max(1, sms) * (o.blocks_per_sm > 0 ? std::min(o.blocks_per_sm, resident) : resident);
    shape.interact_batch = std::min(32, std::max(0, o.interact_batch));
    shape.refill_batch = std::min(32, std::max(0, o.refill_batch));
    shape.woodcock_steps = std::min(64, std::max(0, o.woodcock_steps));

    const auto t0 = std::chrono::steady_clock::now();
    cudaError_t le = cudaSuccess;
    if (h1 > h0)
        le = launchTransportUnpacked(J, h1, counters, shape, s);
    DevCounters c {};
    cudaError_t ce = cudaMemcpyAsync(&c, counters, sizeof(c), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess)
        ce = cudaStreamSynchronize(s);
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (le != cudaSuccess)
        return fail(DXMCG_ERR_CUDA, std::string("transport_run_noalloc: launch: ") + cudaGetErrorString(le));
    if (ce != cudaSuccess)
        return fail(DXMCG_ERR_CUDA, std::string("transport_run_noalloc: ") + cudaGetErrorString(ce));
    if (stats) {
        stats->e_source = c.e_source;
        stats->e_deposited = c.e_deposited;
        stats->e_escaped = c.e_escaped;
        stats->n_histories = c.histories;
        stats->n_missed = c.missed;
        stats->n_visits = c.visits;
        stats->n_voxel_reads = c.visits - c.skipped;
        stats->n_cell_reads = 0; // no cell bounds without a world
        stats->n_photo = c.photo;
        stats->n_compton = c.compton;
        stats->n_rayleigh = c.rayleigh;
        stats->n_cutoff = c.cutoff;
        stats->n_errors = c.errors;
        stats->n_interacted = c.interacted;
        stats->n_crossings = c.crossings;
        stats->n_fluorescence = c.fluorescence;
        stats->kernel_ms = 0.0; // no CUDA events on this path: host wall time of launch + readback below
        stats->total_ms = ms;
        stats->dose_scale = 1.602176634e-10 / (spacing_cm[0] * spacing_cm[1] * spacing_cm[2]);
        stats->calibration = calibration;
        stats->woodcock_steps = o.tracking == DXMCG_TRACK_WOODCOCK ? (shape.woodcock_steps > 0 ? shape.woodcock_steps : 8) : 0;
        stats->two_region = twoRegion ? 1 : 0;
    }
    if (c.error_flags & kErrStepLimit)
        return fail(DXMCG_ERR_DEVICE, "transport_run_noalloc: a history exceeded the step limit");
    if (c.error_flags & kErrRejectLimit)
        return fail(DXMCG_ERR_DEVICE, "transport_run_noalloc: a sampler exceeded its rejection limit");
    return DXMCG_OK;
}
