// capi.cpp -- implementation of the C ABI declared in include/dxmcg.h.
//
// Host side of the engine: world ingest and build (AAVoxelGrid::setData,
// World::build; simulationpipeline.cpp:127-153), the transport driver
// (Transport::operator(); simulationpipeline.cpp:155-171), progress/cancel
// (TransportProgress; :114-120, :234, :261) and the dose readback
// (doseScored(i); :174-231).  There is no CPU transport here: every run goes to
// the device kernels in transport.cu.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dxmcg.h"
#include "denoiser.hpp"
#include "engine.hpp"
#include "jobs.hpp"
#include "physics.hpp"

using namespace dxmcg;

namespace {
thread_local std::string g_error;

int fail(int code, const std::string& msg)
{
    g_error = msg;
    return code;
}

int cudaFail(cudaError_t e, const char* what)
{
    return fail(DXMCG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define DXMCG_CUDA(call)                       \
    do {                                       \
        cudaError_t e_ = (call);               \
        if (e_ != cudaSuccess)                 \
            return cudaFail(e_, #call);        \
    } while (0)

template <class T>
struct DeviceBuffer {
    T* p = nullptr;
    size_t n = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer() { reset(); }
    cudaError_t alloc(size_t count)
    {
        if (count == n && p)
            return cudaSuccess;
        reset();
        const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess)
            n = count;
        else
            p = nullptr;
        return e;
    }
    void reset()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

constexpr double kKeVToMilliGrayGram = 1.602176634e-10; // mGy * g per keV
// histories per launch by default (progress and cancel act between launches): 2^28 is
// about 75 ms on the 256x256x200 torso.  Each launch boundary costs the persistent
// kernel's tail, about 0.23 ms there: one launch per 2^26 histories measured 283.0 ms
// per 1e9 histories, per 2^28 280.5 ms, one launch 279.8 ms.
constexpr int kDefaultChunkLog2 = 28;

// per-beam device inputs of one job
struct JobBuffers {
    DeviceBuffer<DevExposure> exps;
    DeviceBuffer<DevSpectrum> spec;
    DeviceBuffer<DevBowtie> bowtie;
};
} // namespace

int dxmcg::reportError(int code, const std::string& msg) { return fail(code, msg); }

struct dxmcg_progress {
    std::atomic<uint64_t> done { 0 };
    std::atomic<uint64_t> total { 1 };
    std::atomic<int> stop { 0 };
    std::mutex msgMutex;
    std::string message;
    void setMessage(const std::string& m)
    {
        std::lock_guard<std::mutex> l(msgMutex);
        message = m;
    }
};

struct dxmcg_world {
    int device = 0;
    cudaStream_t stream = nullptr;
    int32_t dims[3] {};
    double spacing[3] {};
    size_t N = 0;
    int correction = 1;
    std::vector<dxmcg_material> materials;
    bool hasData = false;
    bool built = false;
    // device
    DeviceBuffer<double> dens64;
    DeviceBuffer<float> dens32;
    DeviceBuffer<uint8_t> mat;
    DeviceBuffer<uint32_t> vox;
    DeviceBuffer<Tally> tally;
    DeviceBuffer<float> tot;
    DeviceBuffer<float4> xs;
    DeviceBuffer<float> maj;
    DeviceBuffer<DevMaterial> mats;
    DeviceBuffer<float> ctab; // Compton angle quantiles per material and energy
    DeviceBuffer<float> rtab; // Rayleigh angle quantiles per material and energy
    DeviceBuffer<DevCounters> counters;
    DeviceBuffer<unsigned> scratch; // rho max bits [256] + error word
    JobBuffers job; // exposures, spectra, bowtie of the last transport_run
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // macro cells for MACRO tracking, built for one cell size at a time
    DeviceBuffer<float> mscale;
    DeviceBuffer<float> mratio;
    int macroB = 0;
    int mc[3] {};
    // Woodcock gather-skip bounds per cell of 8^3 voxels (built with the world)
    DeviceBuffer<float> cbound;
    int ncell[3] {};
    // two-region Woodcock: box of the voxels whose material is neither 0 nor
    // transparent (lo x, y, z, hi x, y, z), and material 0's majorant
    DeviceBuffer<int> boxBuf;
    DeviceBuffer<float> majOut;
    // dose readback staging when the caller's arrays are not pinned host memory
    DeviceBuffer<double> readDose, readVar;
    DeviceBuffer<unsigned long long> readCount;
    int box[6] {};
    bool hasBox = false;
    std::vector<float> hostTot, hostMaj; // FP32 tables as uploaded
    // Woodcock launch hint: stops (real collisions and escapes) per tentative collision
    // of the last run on this world, 0 before the first
    double stopsPerStep = 0.0;
    std::vector<double> rhoMax;
    double historiesScored = 0.0;
    double voxelVolume = 0.0;
};

namespace {

int ensureStream(dxmcg_world* w)
{
    DXMCG_CUDA(cudaSetDevice(w->device));
    if (!w->stream)
        DXMCG_CUDA(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
    if (!w->ev0)
        DXMCG_CUDA(cudaEventCreate(&w->ev0));
    if (!w->ev1)
        DXMCG_CUDA(cudaEventCreate(&w->ev1));
    return DXMCG_OK;
}

// ratio[m] = max over the table energies of total_m(E) / majorant(E), 256 entries
std::vector<float> majorantRatios(const dxmcg_world* w)
{
    const int M = static_cast<int>(w->materials.size());
    std::vector<float> ratio(256, 0.0f);
    for (int m = 0; m < M; ++m) {
        double r = 0;
        for (int i = 0; i < kNE; ++i)
            if (w->hostMaj[i] > 0)
                r = std::max(r, static_cast<double>(w->hostTot[m * kNE + i]) / w->hostMaj[i]);
        ratio[m] = static_cast<float>(r);
    }
    return ratio;
}

// Macro cells of B^3 voxels: ratio[m] (host), then s_c = max over the cell of
// rho * ratio[m] (device, one block per cell).
int ensureMacroCells(dxmcg_world* w, int B)
{
    if (w->macroB == B && w->mscale.p)
        return DXMCG_OK;
    const std::vector<float> ratio = majorantRatios(w);
    for (int a = 0; a < 3; ++a)
        w->mc[a] = (w->dims[a] + B - 1) / B;
    const size_t nc = static_cast<size_t>(w->mc[0]) * w->mc[1] * w->mc[2];
    DXMCG_CUDA(w->mratio.alloc(256));
    DXMCG_CUDA(w->mscale.alloc(nc));
    DXMCG_CUDA(cudaMemcpyAsync(w->mratio.p, ratio.data(), 256 * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    const cudaError_t e = launchMacroScale(w->vox.p, w->dims[0], w->dims[1], w->dims[2], B, w->mc[0], w->mc[1],
        w->mratio.p, reinterpret_cast<unsigned*>(w->mscale.p), w->stream);
    if (e != cudaSuccess)
        return cudaFail(e, "macro-cell kernel");
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    w->macroB = B;
    return DXMCG_OK;
}

// Everything a launch needs for one beam on one world, uploaded into the world's buffers.
// The beam's exposures, spectra and bowtie go to `jb` (the world's own set unless a
// batch passes one of its own).
// The Woodcock gather skip pays where the voxel words do not stay in L2 (129 MB on a
// GB300): measured +3 % on a 420 MB grid and -3 % on a 52 MB one, where the extra
// cell-bound read costs more than the L2-resident voxel reads it saves.
constexpr size_t kGatherSkipBytes = 64ull << 20;

bool gatherSkipFor(const dxmcg_run_options& o, size_t voxelBytes)
{
    if (o.tracking != DXMCG_TRACK_WOODCOCK || o.gather_skip < 0)
        return false;
    return o.gather_skip > 0 || voxelBytes > kGatherSkipBytes;
}

int prepareJob(dxmcg_world* w, const dxmcg_beam& b, const dxmcg_run_options& o, DevJob& J, uint64_t& nHist,
    double& calibration, JobBuffers* jb = nullptr, int gatherSkip = -1, int twoRegion = -1)
{
    if (!jb)
        jb = &w->job;
    HostJob hj;
    std::string err;
    int rc = buildHostJob(b, w->dims, w->spacing, hj, err);
    if (rc != DXMCG_OK)
        return fail(rc, err);
    nHist = hj.nHist;
    rc = calibrationFactor(b, w->correction, o, hj.nHist, true, calibration, err);
    if (rc != DXMCG_OK)
        return fail(rc, err);
    if (calibration != 1.0)
        for (auto& e : hj.exposures)
            e.weight = static_cast<float>(e.weight * calibration);
    DXMCG_CUDA(jb->exps.alloc(hj.exposures.size()));
    DXMCG_CUDA(cudaMemcpyAsync(jb->exps.p, hj.exposures.data(), hj.exposures.size() * sizeof(DevExposure),
        cudaMemcpyHostToDevice, w->stream));
    DXMCG_CUDA(jb->spec.alloc(2));
    DXMCG_CUDA(cudaMemcpyAsync(jb->spec.p, hj.spec, 2 * sizeof(DevSpectrum), cudaMemcpyHostToDevice, w->stream));
    J = DevJob {};
    if (hj.hasBowtie) {
        DXMCG_CUDA(jb->bowtie.alloc(1));
        DXMCG_CUDA(cudaMemcpyAsync(jb->bowtie.p, &hj.bowtie, sizeof(DevBowtie), cudaMemcpyHostToDevice, w->stream));
        J.bowtie = jb->bowtie.p;
    }
    // the host staging must outlive the asynchronous copies
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    fillJobFields(J, b, o, w->dims, w->spacing, w->correction, static_cast<int>(w->materials.size()),
        static_cast<int>(hj.exposures.size()));
    J.vox = w->vox.p;
    J.tot = w->tot.p;
    J.xs = w->xs.p;
    J.maj = w->maj.p;
    J.mats = w->mats.p;
    J.ctab = w->ctab.p;
    J.rtab = w->rtab.p;
    J.tally = w->tally.p;
    J.exps = jb->exps.p;
    J.spec = jb->spec.p;
    // gatherSkip: 1 on, 0 off, -1 decided from this world's size
    const bool skip = gatherSkip < 0 ? gatherSkipFor(o, w->N * sizeof(uint32_t)) : gatherSkip > 0;
    if (o.tracking == DXMCG_TRACK_WOODCOCK && skip && w->cbound.p) {
        J.cbound = w->cbound.p;
        J.cb[0] = w->ncell[0];
        J.cb[1] = w->ncell[1];
    }
    // twoRegion: 1 on, 0 off, -1 decided from this world's box
    const bool two = twoRegion < 0 ? twoRegionFor(o, boxFraction(w->box, w->dims)) : twoRegion > 0;
    if (o.tracking == DXMCG_TRACK_WOODCOCK && two && w->hasBox)
        setTwoRegion(J, w->box, w->spacing, w->majOut.p);
    if (o.tracking == DXMCG_TRACK_MACRO) {
        const int B = o.macro_cell > 0 ? std::min(o.macro_cell, 1024) : 16;
        rc = ensureMacroCells(w, B);
        if (rc != DXMCG_OK)
            return rc;
        J.mscale = w->mscale.p;
        J.mb = B;
        for (int a = 0; a < 3; ++a) {
            J.mc[a] = w->mc[a];
            J.cellL[a] = static_cast<float>(B * w->spacing[a]);
        }
    }
    return DXMCG_OK;
}

// ktrack: the kernel tracking of the instance that will run (kernelTracking)
// Woodcock steps a lane takes per step phase, by default.  A lane stops at a real
// collision or an escape, with probability p per step; the phase's steps are best near
// 1.4 / p, measured on the single-job workloads (p 0.12 on the 256x256x200 torso with
// one region: best 10-12; p 0.28 with two regions there and on the 512x512x400 torso:
// 4-6; p 0.27 on the DX cylinder: 6).  p comes from the world's previous run; 8 before
// the first.
int defaultWoodcockSteps(double stopsPerStep)
{
    if (!(stopsPerStep > 0.0))
        return 8;
    return static_cast<int>(std::lround(std::min(16.0, std::max(4.0, 1.4 / stopsPerStep))));
}

void noteStops(dxmcg_world* w, const DevCounters& c)
{
    const unsigned long long stops = c.photo + c.compton + c.rayleigh + (c.histories - c.missed);
    if (c.visits > 0)
        w->stopsPerStep = static_cast<double>(stops) / static_cast<double>(c.visits);
}

LaunchShape chooseShape(const dxmcg_world* w, const dxmcg_run_options& o, int ktrack, bool batch = false)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, w->device);
    LaunchShape s;
    s.block = o.block_size > 0 ? o.block_size : 256;
    s.block = std::max(32, std::min(256, s.block / 32 * 32));
    // one wave of resident blocks: the kernel is persistent and pulls work from its queue
    const int resident = batch ? transportMaxBlocksPerSMBatch(s.block, ktrack)
                               : transportMaxBlocksPerSM(s.block, ktrack);
    const int per = o.blocks_per_sm > 0 ? std::min(o.blocks_per_sm, resident) : resident;
    s.grid = std::max(1, sms) * per;
    s.interact_batch = std::min(32, std::max(0, o.interact_batch));
    s.refill_batch = std::min(32, std::max(0, o.refill_batch));
    s.woodcock_steps = o.woodcock_steps > 0 ? std::min(64, o.woodcock_steps) : defaultWoodcockSteps(w->stopsPerStep);
    return s;
}

void fillStats(const DevCounters& c, dxmcg_stats* stats)
{
    stats->e_source = c.e_source;
    stats->e_deposited = c.e_deposited;
    stats->e_escaped = c.e_escaped;
    stats->n_histories = c.histories;
    stats->n_missed = c.missed;
    stats->n_visits = c.visits;
    stats->n_voxel_reads = c.visits - c.skipped;
    stats->n_photo = c.photo;
    stats->n_compton = c.compton;
    stats->n_rayleigh = c.rayleigh;
    stats->n_cutoff = c.cutoff;
    stats->n_errors = c.errors;
    stats->n_interacted = c.interacted;
    stats->n_crossings = c.crossings;
    stats->n_fluorescence = c.fluorescence;
}

// the device's error flags as a status (DXMCG_OK when none)
int deviceErrors(const DevCounters& c, const char* what)
{
    if (c.error_flags & kErrStepLimit)
        return fail(DXMCG_ERR_DEVICE, std::string(what) + ": a history exceeded the step limit");
    if (c.error_flags & kErrRejectLimit)
        return fail(DXMCG_ERR_DEVICE, std::string(what) + ": a sampler exceeded its rejection limit");
    return DXMCG_OK;
}

} // namespace

// Several (world, beam) jobs run by one persistent launch over a shared history
// queue; the launch (counter reset + kernel) is a CUDA graph replayed by each run.
// Batches run in one of two ways, both captured once as a CUDA graph and replayed.
// Per job (when the jobs average at least kPerJobHistories): each job is one launch
// of the single-job kernel, on kBatchStreams streams, so that one job's blocks take
// the SMs another job's tail frees.  Shared queue (smaller jobs): one launch of the
// batch kernel over the concatenated history ranges, whose per-lane job descriptors
// cost about 5 % per history against the single-job kernel.
constexpr uint64_t kPerJobHistories = 1ull << 21;
constexpr int kBatchStreams = 4;

struct dxmcg_batch {
    int device = 0;
    int tracking = DXMCG_TRACK_WOODCOCK;
    bool perJob = false;
    std::vector<DevJob> hostJobs;
    std::vector<LaunchShape> jobShapes;
    DeviceBuffer<DevCounters> jobCounters;
    cudaStream_t side[kBatchStreams] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kBatchStreams] = {};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<dxmcg_world*> worlds;
    std::vector<uint64_t> nHist;
    std::vector<double> calibration;
    std::vector<std::unique_ptr<JobBuffers>> inputs;
    DeviceBuffer<DevJob> jobs;
    DeviceBuffer<unsigned long long> offsets;
    DeviceBuffer<DevCounters> counters;
    LaunchShape shape;
    uint64_t total = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool gatherSkip = false;

    dxmcg_batch() = default;
    dxmcg_batch(const dxmcg_batch&) = delete;
    dxmcg_batch& operator=(const dxmcg_batch&) = delete;
    ~dxmcg_batch()
    {
        cudaSetDevice(device);
        if (stream)
            cudaStreamSynchronize(stream);
        if (exec)
            cudaGraphExecDestroy(exec);
        if (graph)
            cudaGraphDestroy(graph);
        if (ev0)
            cudaEventDestroy(ev0);
        if (ev1)
            cudaEventDestroy(ev1);
        if (fork)
            cudaEventDestroy(fork);
        for (int k = 0; k < kBatchStreams; ++k) {
            if (join[k])
                cudaEventDestroy(join[k]);
            if (side[k])
                cudaStreamDestroy(side[k]);
        }
        if (stream)
            cudaStreamDestroy(stream);
    }
};

namespace {
void addCounters(DevCounters& a, const DevCounters& b)
{
    a.histories += b.histories;
    a.missed += b.missed;
    a.visits += b.visits;
    a.photo += b.photo;
    a.compton += b.compton;
    a.rayleigh += b.rayleigh;
    a.cutoff += b.cutoff;
    a.errors += b.errors;
    a.interacted += b.interacted;
    a.crossings += b.crossings;
    a.fluorescence += b.fluorescence;
    a.e_source += b.e_source;
    a.e_escaped += b.e_escaped;
    a.e_deposited += b.e_deposited;
    a.error_flags |= b.error_flags;
    a.skipped += b.skipped;
    a.outer += b.outer;
}
} // namespace

// the segmentation kernel's per-voxel arithmetic, on the host (no contraction into
// fused multiply-adds: the library's host code is compiled with -ffp-contract=off)
void dxmcg::segmentHost(double h, const SegTable& t, uint8_t& m, double& d)
{
    int i = 0;
    while (i < t.nSep && !(h < t.sep[i]))
        ++i;
    m = static_cast<uint8_t>(i);
    const double v = ((t.slope * h) / 1000.0 + t.offset) / t.att[i];
    d = v < 0.0 ? 0.0 : v;
}

// helpers of the segmentation, organ dose table and readout entry points
namespace {
constexpr uint64_t kStreamChunk = 1ull << 25; // voxels per host<->device round trip

// compositions of the two calibration media of the CT number scale
dxmcg_material waterMaterial()
{
    dxmcg_material m {};
    m.n = 2;
    m.Z[0] = 1;
    m.w[0] = 11.19;
    m.Z[1] = 8;
    m.w[1] = 88.81;
    return m;
}
dxmcg_material dryAirMaterial()
{
    dxmcg_material m {};
    m.n = 3;
    m.Z[0] = 7;
    m.w[0] = 75.5;
    m.Z[1] = 8;
    m.w[1] = 23.2;
    m.Z[2] = 18;
    m.w[2] = 1.3;
    return m;
}

bool sameTable(const SegTable& a, const SegTable& b)
{
    return a.nSep == b.nSep && a.slope == b.slope && a.offset == b.offset
        && std::memcmp(a.sep, b.sep, sizeof(double) * a.nSep) == 0
        && std::memcmp(a.att, b.att, sizeof(double) * (a.nSep + 1)) == 0;
}

// The integer-CT-number lookup table of a segmentation table on the current device,
// kept per thread until the table changes.
struct SegLut {
    int device = -1;
    SegTable key {};
    DeviceBuffer<double> d;
    DeviceBuffer<uint8_t> m;
};
int segLut(const SegTable& t, const double*& lutD, const uint8_t*& lutM)
{
    thread_local SegLut cache;
    int dev = 0;
    DXMCG_CUDA(cudaGetDevice(&dev));
    if (cache.device != dev || !sameTable(cache.key, t)) {
        std::vector<double> hd(kSegLutSize);
        std::vector<uint8_t> hm(kSegLutSize);
        for (int k = 0; k < kSegLutSize; ++k)
            segmentHost(static_cast<double>(kSegLutMin + k), t, hm[k], hd[k]);
        if (cache.device != dev) {
            cache.d.reset();
            cache.m.reset();
        }
        DXMCG_CUDA(cache.d.alloc(kSegLutSize));
        DXMCG_CUDA(cache.m.alloc(kSegLutSize));
        DXMCG_CUDA(cudaMemcpy(cache.d.p, hd.data(), kSegLutSize * sizeof(double), cudaMemcpyHostToDevice));
        DXMCG_CUDA(cudaMemcpy(cache.m.p, hm.data(), kSegLutSize, cudaMemcpyHostToDevice));
        cache.device = dev;
        cache.key = t;
    }
    lutD = cache.d.p;
    lutM = cache.m.p;
    return DXMCG_OK;
}

int toSegTable(const dxmcg_segmentation* t, SegTable& s)
{
    if (!t || t->n_materials < 1 || t->n_materials > DXMCG_MAX_SEG_MATERIALS)
        return fail(DXMCG_ERR_ARGUMENT, "ct_segment: bad segmentation table");
    s = SegTable {};
    s.nSep = t->n_materials - 1;
    s.slope = t->water_attenuation * t->water_density - t->air_attenuation * t->air_density;
    s.offset = t->water_attenuation * t->water_density;
    for (int i = 0; i < s.nSep; ++i)
        s.sep[i] = t->separator[i];
    for (int i = 0; i < t->n_materials; ++i)
        s.att[i] = t->attenuation[i];
    return DXMCG_OK;
}

void organRows(const std::vector<unsigned long long>& cnt, const std::vector<double>& rho,
    const std::vector<double>& e, double voxelVolume, int nOrgans, dxmcg_organ_dose* out)
{
    for (int i = 0; i < nOrgans; ++i) {
        out[i] = dxmcg_organ_dose {};
        if (cnt[i] == 0)
            continue;
        out[i].n_voxels = cnt[i];
        out[i].volume_cm3 = static_cast<double>(cnt[i]) * voxelVolume;
        out[i].mass_g = voxelVolume * rho[i];
        out[i].dose = out[i].mass_g > 0.0 ? e[i] / out[i].mass_g : 0.0;
    }
}

// per-organ sums on the device: count, sum of density, sum of dose x mass
struct OrganSums {
    DeviceBuffer<unsigned long long> cnt;
    DeviceBuffer<double> rho, e;
    int alloc(cudaStream_t s)
    {
        DXMCG_CUDA(cnt.alloc(256));
        DXMCG_CUDA(rho.alloc(256));
        DXMCG_CUDA(e.alloc(256));
        DXMCG_CUDA(cudaMemsetAsync(cnt.p, 0, 256 * sizeof(unsigned long long), s));
        DXMCG_CUDA(cudaMemsetAsync(rho.p, 0, 256 * sizeof(double), s));
        DXMCG_CUDA(cudaMemsetAsync(e.p, 0, 256 * sizeof(double), s));
        return DXMCG_OK;
    }
    int read(double voxelVolume, int nOrgans, dxmcg_organ_dose* out, cudaStream_t s)
    {
        std::vector<unsigned long long> c(256);
        std::vector<double> r(256), en(256);
        DXMCG_CUDA(cudaMemcpyAsync(c.data(), cnt.p, 256 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        DXMCG_CUDA(cudaMemcpyAsync(r.data(), rho.p, 256 * sizeof(double), cudaMemcpyDeviceToHost, s));
        DXMCG_CUDA(cudaMemcpyAsync(en.data(), e.p, 256 * sizeof(double), cudaMemcpyDeviceToHost, s));
        DXMCG_CUDA(cudaStreamSynchronize(s));
        organRows(c, r, en, voxelVolume, nOrgans, out);
        return DXMCG_OK;
    }
};

// the calling thread's sums on its current device, kept between calls (a table is a
// few hundred bytes; allocating it per call would put a cudaFree in every call)
OrganSums& organSums()
{
    thread_local std::map<int, std::unique_ptr<OrganSums>> perDevice;
    int dev = 0;
    cudaGetDevice(&dev);
    auto& p = perDevice[dev];
    if (!p)
        p = std::make_unique<OrganSums>();
    return *p;
}

int checkOrganArgs(const double* spacing, int nOrgans, const dxmcg_organ_dose* out, double& V)
{
    if (!spacing || !out || nOrgans < 1 || nOrgans > 256)
        return fail(DXMCG_ERR_ARGUMENT, "organ_dose_table: need spacing, 1..256 organs and an output array");
    V = spacing[0] * spacing[1] * spacing[2];
    if (!(V > 0.0))
        return fail(DXMCG_ERR_ARGUMENT, "organ_dose_table: spacing must be positive");
    return DXMCG_OK;
}

int currentDevice()
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1)
        return fail(DXMCG_ERR_NO_DEVICE, "no CUDA device");
    return DXMCG_OK;
}
} // namespace

// ============================================================================ C ABI
extern "C" {

DXMCG_API int dxmcg_version(void) { return DXMCG_VERSION; }

DXMCG_API const char* dxmcg_last_error(void) { return g_error.c_str(); }

DXMCG_API int dxmcg_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess)
        return 0;
    return n;
}

DXMCG_API int dxmcg_set_device(int device)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1)
        return fail(DXMCG_ERR_NO_DEVICE, "set_device: no CUDA device");
    if (device < 0 || device >= n)
        return fail(DXMCG_ERR_ARGUMENT, "set_device: no such device");
    DXMCG_CUDA(cudaSetDevice(device));
    return DXMCG_OK;
}

DXMCG_API int dxmcg_material_attenuation(const dxmcg_material* m, int correction, int n, const double* energies,
    double* photo, double* incoherent, double* coherent)
{
    if (!m || !validComposition(*m) || n < 0 || (n > 0 && (!energies || !photo || !incoherent || !coherent)))
        return fail(DXMCG_ERR_ARGUMENT, "material_attenuation: bad arguments");
    for (int i = 0; i < n; ++i) {
        const auto a = attenuation(*m, correction, energies[i]);
        photo[i] = a.photo;
        incoherent[i] = a.incoherent;
        coherent[i] = a.coherent;
    }
    return DXMCG_OK;
}

DXMCG_API int dxmcg_tube_spectrum(double kvp, double anode_angle_deg, int n_filters, const int32_t* filter_Z,
    const double* filter_mm, double* energies, double* weights, int cap, int* n_out)
{
    if (n_filters < 0 || n_filters > 8 || (n_filters > 0 && (!filter_Z || !filter_mm)))
        return fail(DXMCG_ERR_ARGUMENT, "tube_spectrum: bad filters");
    const auto s = tubeSpectrum(kvp, anode_angle_deg, n_filters, filter_Z, filter_mm);
    if (s.energy.empty())
        return fail(DXMCG_ERR_ARGUMENT, "tube_spectrum: tube voltage out of range");
    if (n_out)
        *n_out = static_cast<int>(s.energy.size());
    if (!energies || !weights)
        return DXMCG_OK;
    if (cap < static_cast<int>(s.energy.size()))
        return fail(DXMCG_ERR_CAPACITY, "tube_spectrum: output too small");
    std::copy(s.energy.begin(), s.energy.end(), energies);
    std::copy(s.weight.begin(), s.weight.end(), weights);
    return DXMCG_OK;
}

DXMCG_API int dxmcg_tube_mean_energy(double kvp, int n_filters, const int32_t* filter_Z, const double* filter_mm,
    double* mean_kev)
{
    const auto s = tubeSpectrum(kvp, 12.0, n_filters, filter_Z, filter_mm);
    if (s.energy.empty() || !mean_kev)
        return fail(DXMCG_ERR_ARGUMENT, "tube_mean_energy: bad arguments");
    *mean_kev = tubeMeanEnergy(s);
    return DXMCG_OK;
}

DXMCG_API int dxmcg_tube_al_hvl(double kvp, int n_filters, const int32_t* filter_Z, const double* filter_mm,
    double* hvl_mm)
{
    const auto s = tubeSpectrum(kvp, 12.0, n_filters, filter_Z, filter_mm);
    if (s.energy.empty() || !hvl_mm)
        return fail(DXMCG_ERR_ARGUMENT, "tube_al_hvl: bad arguments");
    *hvl_mm = tubeAlHalfValueLayer(s);
    return DXMCG_OK;
}

DXMCG_API int dxmcg_beam_exposures(const dxmcg_beam* beam, dxmcg_exposure* out, int cap, int* n_out)
{
    if (!beam)
        return fail(DXMCG_ERR_ARGUMENT, "beam_exposures: null beam");
    std::vector<dxmcg_exposure> ex;
    const int rc = expandExposures(*beam, ex);
    if (rc != DXMCG_OK)
        return fail(rc, "beam_exposures: invalid beam geometry");
    if (n_out)
        *n_out = static_cast<int>(ex.size());
    if (!out)
        return DXMCG_OK;
    if (cap < static_cast<int>(ex.size()))
        return fail(DXMCG_ERR_CAPACITY, "beam_exposures: output too small");
    std::copy(ex.begin(), ex.end(), out);
    return DXMCG_OK;
}

DXMCG_API int dxmcg_physics_load(const char* path)
{
    if (!path)
        return fail(DXMCG_ERR_ARGUMENT, "physics_load: null path");
    std::string err;
    const int rc = loadPhysicsTable(path, err);
    return rc == DXMCG_OK ? rc : fail(rc, "physics_load: " + err);
}

DXMCG_API int dxmcg_physics_reset(void)
{
    resetPhysicsTable();
    return DXMCG_OK;
}

DXMCG_API int dxmcg_physics_write(const char* path, int n_elements, const int32_t* Z)
{
    if (!path || n_elements < 0 || (n_elements > 0 && !Z))
        return fail(DXMCG_ERR_ARGUMENT, "physics_write: bad arguments");
    std::string err;
    const int rc = writePhysicsTable(path, n_elements, Z, err);
    return rc == DXMCG_OK ? rc : fail(rc, "physics_write: " + err);
}

DXMCG_API int dxmcg_beam_calibration(const dxmcg_beam* beam, int correction, const dxmcg_run_options* opts,
    double* factor)
{
    if (!beam || !factor)
        return fail(DXMCG_ERR_ARGUMENT, "beam_calibration: null argument");
    if (correction < 0 || correction > 2)
        return fail(DXMCG_ERR_ARGUMENT, "beam_calibration: correction must be 0, 1 or 2");
    std::vector<dxmcg_exposure> ex;
    if (expandExposures(*beam, ex) != DXMCG_OK || ex.empty())
        return fail(DXMCG_ERR_ARGUMENT, "beam_calibration: invalid beam geometry");
    dxmcg_run_options o {};
    o.seed = 1;
    if (opts)
        o = *opts;
    const uint64_t nHist = static_cast<uint64_t>(ex.size()) * beam->particles_per_exposure;
    std::string err;
    const int rc = calibrationFactor(*beam, correction, o, nHist, true, *factor, err);
    if (rc != DXMCG_OK)
        return fail(rc, "beam_calibration: " + err);
    return DXMCG_OK;
}

DXMCG_API int dxmcg_world_create(const int32_t dims[3], const double spacing_cm[3], const dxmcg_material* materials,
    int n_materials, int correction, dxmcg_world** out)
{
    if (!out)
        return fail(DXMCG_ERR_ARGUMENT, "world_create: null output");
    *out = nullptr;
    if (!dims || !spacing_cm || !materials || n_materials < 1 || n_materials > DXMCG_MAX_MATERIALS)
        return fail(DXMCG_ERR_ARGUMENT, "world_create: need 1..255 materials");
    uint64_t N = 1;
    for (int a = 0; a < 3; ++a) {
        if (dims[a] < 1 || !(spacing_cm[a] > 0) || !std::isfinite(spacing_cm[a]))
            return fail(DXMCG_ERR_ARGUMENT, "world_create: dimensions and spacing must be positive");
        N *= static_cast<uint64_t>(dims[a]);
    }
    if (N >= (1ull << 32))
        return fail(DXMCG_ERR_ARGUMENT, "world_create: more than 2^32-1 voxels");
    for (int m = 0; m < n_materials; ++m)
        if (!validComposition(materials[m]))
            return fail(DXMCG_ERR_ARGUMENT, "world_create: invalid material composition " + std::to_string(m));
    if (correction < 0 || correction > 2)
        return fail(DXMCG_ERR_ARGUMENT, "world_create: correction must be 0, 1 or 2");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
        return fail(DXMCG_ERR_NO_DEVICE, "world_create: no CUDA device");
    auto* w = new dxmcg_world();
    cudaGetDevice(&w->device);
    for (int a = 0; a < 3; ++a) {
        w->dims[a] = dims[a];
        w->spacing[a] = spacing_cm[a];
    }
    w->N = static_cast<size_t>(N);
    w->voxelVolume = spacing_cm[0] * spacing_cm[1] * spacing_cm[2];
    w->correction = correction;
    w->materials.assign(materials, materials + n_materials);
    const int rc = ensureStream(w);
    if (rc != DXMCG_OK) {
        dxmcg_world_destroy(w);
        return rc;
    }
    *out = w;
    return DXMCG_OK;
}

static int setData(dxmcg_world* w, const double* d64, const float* d32, const uint8_t* material)
{
    if (!w || (!d64 && !d32) || !material)
        return fail(DXMCG_ERR_ARGUMENT, "world_set_data: null argument");
    DXMCG_CUDA(cudaSetDevice(w->device));
    DXMCG_CUDA(w->mat.alloc(w->N));
    if (d64) {
        w->dens32.reset();
        DXMCG_CUDA(w->dens64.alloc(w->N));
        DXMCG_CUDA(cudaMemcpyAsync(w->dens64.p, d64, w->N * sizeof(double), cudaMemcpyHostToDevice, w->stream));
    } else {
        w->dens64.reset();
        DXMCG_CUDA(w->dens32.alloc(w->N));
        DXMCG_CUDA(cudaMemcpyAsync(w->dens32.p, d32, w->N * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    }
    DXMCG_CUDA(cudaMemcpyAsync(w->mat.p, material, w->N, cudaMemcpyHostToDevice, w->stream));
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    w->hasData = true;
    w->built = false;
    return DXMCG_OK;
}

DXMCG_API int dxmcg_world_set_data(dxmcg_world* w, const double* density, const uint8_t* material)
{
    return setData(w, density, nullptr, material);
}

DXMCG_API int dxmcg_world_set_data_f32(dxmcg_world* w, const float* density, const uint8_t* material)
{
    return setData(w, nullptr, density, material);
}

DXMCG_API int dxmcg_world_build(dxmcg_world* w)
{
    if (!w || !w->hasData)
        return fail(DXMCG_ERR_STATE, "world_build: setData first");
    DXMCG_CUDA(cudaSetDevice(w->device));
    const int M = static_cast<int>(w->materials.size());
    DXMCG_CUDA(w->vox.alloc(w->N));
    DXMCG_CUDA(w->scratch.alloc(257));
    DXMCG_CUDA(cudaMemsetAsync(w->scratch.p, 0, 257 * sizeof(unsigned), w->stream));
    cudaError_t e = launchPack(w->dens64.p, w->dens32.p, w->mat.p, w->vox.p, w->N, M, w->scratch.p,
        w->scratch.p + 256, w->stream);
    if (e != cudaSuccess)
        return cudaFail(e, "pack kernel");
    unsigned host[257];
    DXMCG_CUDA(cudaMemcpyAsync(host, w->scratch.p, sizeof(host), cudaMemcpyDeviceToHost, w->stream));
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    if (host[256] & kErrBadMaterial)
        return fail(DXMCG_ERR_ARGUMENT, "world_build: a voxel's material index is >= the number of materials");
    if (host[256] & kErrBadDensity)
        return fail(DXMCG_ERR_ARGUMENT, "world_build: negative or non-finite density");
    // the staging arrays stay allocated: a caller that sets data and builds again each
    // run (a new patient, the same grid) then allocates nothing

    w->rhoMax.assign(M, 0.0);
    for (int m = 0; m < M; ++m) {
        float f;
        std::memcpy(&f, &host[m], 4);
        w->rhoMax[m] = f;
    }
    std::vector<float> tot(static_cast<size_t>(M) * kNE);
    std::vector<float4> xs(static_cast<size_t>(M) * kNE);
    std::vector<float> majf(kNE);
    std::vector<DevMaterial> dm(M);
    buildDeviceTables(w->materials.data(), M, w->correction, w->rhoMax.data(), tot.data(), xs.data(), majf.data(),
        dm.data());
    w->hostTot = tot;
    w->hostMaj = majf;
    w->macroB = 0;
    DXMCG_CUDA(w->tot.alloc(tot.size()));
    DXMCG_CUDA(w->xs.alloc(xs.size()));
    DXMCG_CUDA(w->maj.alloc(kNE));
    DXMCG_CUDA(w->mats.alloc(M));
    DXMCG_CUDA(w->counters.alloc(1));
    DXMCG_CUDA(w->tally.alloc(w->N));
    DXMCG_CUDA(cudaMemcpyAsync(w->tot.p, tot.data(), tot.size() * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    DXMCG_CUDA(cudaMemcpyAsync(w->xs.p, xs.data(), xs.size() * sizeof(float4), cudaMemcpyHostToDevice, w->stream));
    DXMCG_CUDA(cudaMemcpyAsync(w->maj.p, majf.data(), kNE * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    DXMCG_CUDA(cudaMemcpyAsync(w->mats.p, dm.data(), M * sizeof(DevMaterial), cudaMemcpyHostToDevice, w->stream));
    std::vector<float> ctab(static_cast<size_t>(M) * kNE * kCTabK);
    buildComptonAngleTables(w->materials.data(), M, w->correction, ctab.data());
    DXMCG_CUDA(w->ctab.alloc(ctab.size()));
    DXMCG_CUDA(cudaMemcpyAsync(w->ctab.p, ctab.data(), ctab.size() * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    std::vector<float> rtab(static_cast<size_t>(M) * kNE * kCTabK);
    buildRayleighAngleTables(w->materials.data(), M, rtab.data());
    DXMCG_CUDA(w->rtab.alloc(rtab.size()));
    DXMCG_CUDA(cudaMemcpyAsync(w->rtab.p, rtab.data(), rtab.size() * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    DXMCG_CUDA(cudaMemsetAsync(w->tally.p, 0, w->N * sizeof(Tally), w->stream));
    // gather-skip bounds of the Woodcock step
    {
        const std::vector<float> ratio = majorantRatios(w);
        for (int a = 0; a < 3; ++a)
            w->ncell[a] = (w->dims[a] + kCellEdge - 1) / kCellEdge;
        const size_t nc = static_cast<size_t>(w->ncell[0]) * w->ncell[1] * w->ncell[2];
        DXMCG_CUDA(w->mratio.alloc(256));
        DXMCG_CUDA(w->cbound.alloc(nc));
        DXMCG_CUDA(cudaMemcpyAsync(w->mratio.p, ratio.data(), 256 * sizeof(float), cudaMemcpyHostToDevice, w->stream));
        e = launchCellBound(w->vox.p, w->dims[0], w->dims[1], w->dims[2], w->ncell[0], w->ncell[1], w->ncell[2],
            w->mratio.p, w->cbound.p, w->stream);
        if (e != cudaSuccess)
            return cudaFail(e, "cell-bound kernel");
    }
    // two-region box and material 0's majorant
    {
        const int init[6] = { INT_MAX, INT_MAX, INT_MAX, -1, -1, -1 };
        DXMCG_CUDA(w->boxBuf.alloc(6));
        DXMCG_CUDA(cudaMemcpyAsync(w->boxBuf.p, init, sizeof(init), cudaMemcpyHostToDevice, w->stream));
        e = launchMaterialBox(w->vox.p, w->dims[0], w->dims[1], w->dims[2], w->boxBuf.p, w->stream);
        if (e != cudaSuccess)
            return cudaFail(e, "material-box kernel");
        DXMCG_CUDA(cudaMemcpyAsync(w->box, w->boxBuf.p, sizeof(w->box), cudaMemcpyDeviceToHost, w->stream));
        std::vector<float> mo(kNE);
        buildBackgroundMajorant(tot.data(), w->rhoMax[0], mo.data());
        DXMCG_CUDA(w->majOut.alloc(kNE));
        DXMCG_CUDA(cudaMemcpyAsync(w->majOut.p, mo.data(), kNE * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    }
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    w->hasBox = twoRegionBox(w->box, w->dims);
    w->historiesScored = 0.0;
    w->built = true;
    return DXMCG_OK;
}

DXMCG_API void dxmcg_world_destroy(dxmcg_world* w)
{
    if (!w)
        return;
    cudaSetDevice(w->device);
    if (w->stream)
        cudaStreamSynchronize(w->stream);
    if (w->ev0)
        cudaEventDestroy(w->ev0);
    if (w->ev1)
        cudaEventDestroy(w->ev1);
    if (w->stream)
        cudaStreamDestroy(w->stream);
    delete w;
}

DXMCG_API int dxmcg_world_clear_tally(dxmcg_world* w)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "world_clear_tally: world not built");
    DXMCG_CUDA(cudaSetDevice(w->device));
    DXMCG_CUDA(cudaMemsetAsync(w->tally.p, 0, w->N * sizeof(Tally), w->stream));
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    w->historiesScored = 0.0;
    return DXMCG_OK;
}

DXMCG_API int dxmcg_world_read_tally(dxmcg_world* w, double* energy, double* energy2, uint64_t* count)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "world_read_tally: world not built");
    DXMCG_CUDA(cudaSetDevice(w->device));
    std::vector<Tally> t(w->N);
    DXMCG_CUDA(cudaMemcpyAsync(t.data(), w->tally.p, w->N * sizeof(Tally), cudaMemcpyDeviceToHost, w->stream));
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    for (size_t i = 0; i < w->N; ++i) {
        if (energy)
            energy[i] = t[i].e;
        if (energy2)
            energy2[i] = t[i].e2;
        if (count)
            count[i] = t[i].n;
    }
    return DXMCG_OK;
}

namespace {
// Device address of caller memory the GPU can write directly: pinned host memory
// (mapped under unified addressing) or device memory; nullptr for pageable memory.
void* deviceWritable(void* p)
{
    if (!p)
        return nullptr;
    cudaPointerAttributes a {};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
        return p;
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}
} // namespace

DXMCG_API int dxmcg_world_read_dose(dxmcg_world* w, double* dose, double* variance, uint64_t* count)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "world_read_dose: world not built");
    DXMCG_CUDA(cudaSetDevice(w->device));
    // The finalize kernel writes straight into arrays the GPU can address (pinned host
    // memory over the host link, or device memory); the others are staged in the
    // world's readback buffers and copied.
    double* dd = static_cast<double*>(deviceWritable(dose));
    double* dv = static_cast<double*>(deviceWritable(variance));
    auto* dc = static_cast<unsigned long long*>(deviceWritable(count));
    if (dose && !dd) {
        DXMCG_CUDA(w->readDose.alloc(w->N));
        dd = w->readDose.p;
    }
    if (variance && !dv) {
        DXMCG_CUDA(w->readVar.alloc(w->N));
        dv = w->readVar.p;
    }
    if (count && !dc) {
        DXMCG_CUDA(w->readCount.alloc(w->N));
        dc = w->readCount.p;
    }
    cudaError_t e = launchFinalize(w->tally.p, w->vox.p, w->N, kKeVToMilliGrayGram / w->voxelVolume,
        w->historiesScored, dd, dv, dc, w->stream);
    if (e != cudaSuccess)
        return cudaFail(e, "finalize kernel");
    if (dose && dd == w->readDose.p)
        DXMCG_CUDA(cudaMemcpyAsync(dose, dd, w->N * sizeof(double), cudaMemcpyDeviceToHost, w->stream));
    if (variance && dv == w->readVar.p)
        DXMCG_CUDA(cudaMemcpyAsync(variance, dv, w->N * sizeof(double), cudaMemcpyDeviceToHost, w->stream));
    if (count && dc == w->readCount.p)
        DXMCG_CUDA(cudaMemcpyAsync(count, dc, w->N * sizeof(uint64_t), cudaMemcpyDeviceToHost, w->stream));
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    return DXMCG_OK;
}

DXMCG_API int dxmcg_world_tables(dxmcg_world* w, int material, float* xs4, float* majorant)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "world_tables: world not built");
    if (material < 0 || material >= static_cast<int>(w->materials.size()))
        return fail(DXMCG_ERR_ARGUMENT, "world_tables: bad material");
    DXMCG_CUDA(cudaSetDevice(w->device));
    if (xs4)
        DXMCG_CUDA(cudaMemcpy(xs4, w->xs.p + static_cast<size_t>(material) * kNE, kNE * sizeof(float4),
            cudaMemcpyDeviceToHost));
    if (majorant)
        DXMCG_CUDA(cudaMemcpy(majorant, w->maj.p, kNE * sizeof(float), cudaMemcpyDeviceToHost));
    return DXMCG_OK;
}

DXMCG_API int dxmcg_world_packed_density(dxmcg_world* w, float* density, uint8_t* material)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "world_packed_density: world not built");
    DXMCG_CUDA(cudaSetDevice(w->device));
    std::vector<uint32_t> v(w->N);
    DXMCG_CUDA(cudaMemcpy(v.data(), w->vox.p, w->N * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < w->N; ++i) {
        if (density) {
            const uint32_t b = v[i] & 0xffffff00u;
            std::memcpy(&density[i], &b, 4);
        }
        if (material)
            material[i] = static_cast<uint8_t>(v[i] & 0xffu);
    }
    return DXMCG_OK;
}

DXMCG_API int dxmcg_transport_run(dxmcg_world* w, const dxmcg_beam* beam, const dxmcg_run_options* opts,
    dxmcg_progress* progress, dxmcg_stats* stats)
{
    const auto t0 = std::chrono::steady_clock::now();
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "transport_run: world not built");
    if (!beam)
        return fail(DXMCG_ERR_ARGUMENT, "transport_run: null beam");
    dxmcg_run_options o {};
    o.seed = 1;
    if (opts)
        o = *opts;
    if (o.tracking != DXMCG_TRACK_WOODCOCK && o.tracking != DXMCG_TRACK_SIDDON && o.tracking != DXMCG_TRACK_MACRO)
        return fail(DXMCG_ERR_ARGUMENT, "transport_run: unknown tracking mode");
    DXMCG_CUDA(cudaSetDevice(w->device));
    DevJob J;
    uint64_t nHist = 0;
    double calibration = 1.0;
    int rc = prepareJob(w, *beam, o, J, nHist, calibration);
    if (rc != DXMCG_OK)
        return rc;
    DXMCG_CUDA(cudaSetDevice(w->device)); // the CTDI calibration may have run another world
    const uint64_t h0 = std::min<uint64_t>(o.hist_begin, nHist);
    const uint64_t h1 = o.hist_end == 0 ? nHist : std::min<uint64_t>(o.hist_end, nHist);
    if (progress) {
        progress->total.store(std::max<uint64_t>(h1 - h0, 1));
        progress->done.store(0);
        progress->setMessage("Simulating");
    }
    const LaunchShape shape = chooseShape(w, o, kernelTracking(J));
    const int chunkLog2 = o.chunk_histories_log2 > 0 ? std::min(o.chunk_histories_log2, 40) : kDefaultChunkLog2;
    const uint64_t chunk = 1ull << chunkLog2;
    DevCounters zero {};
    DXMCG_CUDA(cudaMemcpyAsync(w->counters.p, &zero, sizeof(zero), cudaMemcpyHostToDevice, w->stream));
    float kernelMs = 0.0f;
    bool cancelled = false;
    for (uint64_t a = h0; a < h1; a += chunk) {
        if (progress && progress->stop.load()) {
            cancelled = true;
            break;
        }
        const uint64_t b = std::min(h1, a + chunk);
        const unsigned long long head = a;
        DXMCG_CUDA(cudaMemcpyAsync(&w->counters.p->next, &head, sizeof(head), cudaMemcpyHostToDevice, w->stream));
        DXMCG_CUDA(cudaEventRecord(w->ev0, w->stream));
        cudaError_t e = launchTransport(J, b, w->counters.p, shape, w->stream);
        if (e != cudaSuccess)
            return cudaFail(e, "transport kernel launch");
        DXMCG_CUDA(cudaEventRecord(w->ev1, w->stream));
        DXMCG_CUDA(cudaEventSynchronize(w->ev1));
        float ms = 0;
        DXMCG_CUDA(cudaEventElapsedTime(&ms, w->ev0, w->ev1));
        kernelMs += ms;
        if (progress)
            progress->done.store(b - h0);
    }
    DevCounters c {};
    DXMCG_CUDA(cudaMemcpyAsync(&c, w->counters.p, sizeof(c), cudaMemcpyDeviceToHost, w->stream));
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    w->historiesScored += static_cast<double>(c.histories);
    if (o.tracking == DXMCG_TRACK_WOODCOCK)
        noteStops(w, c);
    if (stats) {
        stats->e_source = c.e_source;
        stats->e_deposited = c.e_deposited;
        stats->e_escaped = c.e_escaped;
        stats->n_histories = c.histories;
        stats->n_missed = c.missed;
        stats->n_visits = c.visits;
        stats->n_voxel_reads = c.visits - c.skipped;
        stats->n_cell_reads = J.cbound ? c.visits - c.outer : 0;
        stats->n_photo = c.photo;
        stats->n_compton = c.compton;
        stats->n_rayleigh = c.rayleigh;
        stats->n_cutoff = c.cutoff;
        stats->n_errors = c.errors;
        stats->n_interacted = c.interacted;
        stats->n_crossings = c.crossings;
        stats->n_fluorescence = c.fluorescence;
        stats->kernel_ms = kernelMs;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->dose_scale = kKeVToMilliGrayGram / w->voxelVolume;
        stats->calibration = calibration;
        stats->woodcock_steps = o.tracking == DXMCG_TRACK_WOODCOCK ? shape.woodcock_steps : 0;
        stats->two_region = J.boxOn;
    }
    if (progress)
        progress->setMessage(cancelled ? "Cancelled" : "Done");
    if (c.error_flags & kErrStepLimit)
        return fail(DXMCG_ERR_DEVICE, "transport: a history exceeded the step limit");
    if (c.error_flags & kErrRejectLimit)
        return fail(DXMCG_ERR_DEVICE, "transport: a sampler exceeded its rejection limit");
    if (cancelled)
        return fail(DXMCG_ERR_CANCELLED, "transport: cancelled");
    return DXMCG_OK;
}

DXMCG_API int dxmcg_batch_create(int n_jobs, dxmcg_world* const* worlds, const dxmcg_beam* beams,
    const dxmcg_run_options* opts, dxmcg_batch** out)
{
    if (!out)
        return fail(DXMCG_ERR_ARGUMENT, "batch_create: null out");
    *out = nullptr;
    if (n_jobs < 1 || !worlds || !beams || !opts)
        return fail(DXMCG_ERR_ARGUMENT, "batch_create: need n_jobs >= 1 worlds, beams and options");
    const int tracking = opts[0].tracking;
    if (tracking != DXMCG_TRACK_WOODCOCK && tracking != DXMCG_TRACK_SIDDON && tracking != DXMCG_TRACK_MACRO)
        return fail(DXMCG_ERR_ARGUMENT, "batch_create: unknown tracking mode");
    for (int j = 0; j < n_jobs; ++j) {
        if (!worlds[j] || !worlds[j]->built)
            return fail(DXMCG_ERR_STATE, "batch_create: job " + std::to_string(j) + ": world not built");
        if (worlds[j]->device != worlds[0]->device)
            return fail(DXMCG_ERR_ARGUMENT, "batch_create: all worlds must be on one device");
        if (opts[j].tracking != tracking)
            return fail(DXMCG_ERR_ARGUMENT, "batch_create: all jobs must use one tracking mode");
        if (opts[j].hist_begin != 0 || opts[j].hist_end != 0)
            return fail(DXMCG_ERR_ARGUMENT, "batch_create: jobs run whole beams (hist_begin/hist_end must be 0)");
    }
    auto b = std::make_unique<dxmcg_batch>();
    b->device = worlds[0]->device;
    b->tracking = tracking;
    DXMCG_CUDA(cudaSetDevice(b->device));
    DXMCG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    DXMCG_CUDA(cudaEventCreate(&b->ev0));
    DXMCG_CUDA(cudaEventCreate(&b->ev1));
    std::vector<DevJob> J(n_jobs);
    std::vector<unsigned long long> off(n_jobs + 1, 0ull);
    // one gather-skip decision for the whole batch, from opts[0] and the voxel words
    // of all its (distinct) worlds: they share L2 during the launch
    size_t voxelBytes = 0;
    for (int j = 0; j < n_jobs; ++j) {
        bool seen = false;
        for (int i = 0; i < j; ++i)
            seen = seen || worlds[i] == worlds[j];
        if (!seen)
            voxelBytes += worlds[j]->N * sizeof(uint32_t);
    }
    b->gatherSkip = gatherSkipFor(opts[0], voxelBytes);
    for (int j = 0; j < n_jobs; ++j) {
        b->inputs.push_back(std::make_unique<JobBuffers>());
        uint64_t n = 0;
        double cal = 1.0;
        const int rc = prepareJob(worlds[j], beams[j], opts[j], J[j], n, cal, b->inputs.back().get(),
            b->gatherSkip ? 1 : 0);
        if (rc != DXMCG_OK)
            return rc;
        b->worlds.push_back(worlds[j]);
        b->nHist.push_back(n);
        b->calibration.push_back(cal);
        off[j + 1] = off[j] + n;
    }
    // a world's macro cells are rebuilt when a later job asks for another size
    if (tracking == DXMCG_TRACK_MACRO)
        for (int j = 0; j < n_jobs; ++j)
            if (J[j].mb != worlds[j]->macroB || J[j].mscale != worlds[j]->mscale.p)
                return fail(DXMCG_ERR_ARGUMENT, "batch_create: jobs on one world must use one macro_cell");
    b->total = off[n_jobs];
    DXMCG_CUDA(cudaSetDevice(b->device));
    DXMCG_CUDA(b->jobs.alloc(n_jobs));
    DXMCG_CUDA(b->offsets.alloc(n_jobs + 1));
    DXMCG_CUDA(b->counters.alloc(1));
    DXMCG_CUDA(cudaMemcpyAsync(b->jobs.p, J.data(), n_jobs * sizeof(DevJob), cudaMemcpyHostToDevice, b->stream));
    DXMCG_CUDA(cudaMemcpyAsync(b->offsets.p, off.data(), off.size() * sizeof(unsigned long long),
        cudaMemcpyHostToDevice, b->stream));
    DXMCG_CUDA(cudaStreamSynchronize(b->stream));
    // the occupancy query also loads the kernel, so the later graph capture loads nothing
    // Woodcock jobs run the two-region instance when any of them has a box; in it, a
    // job without one (boxOn 0) never leaves the first region
    for (int j = 0; j < n_jobs; ++j)
        if (kernelTracking(J[j]) == kTrackWoodcockBox)
            b->tracking = kTrackWoodcockBox;
    b->shape = chooseShape(worlds[0], opts[0], b->tracking, true);
    b->perJob = b->total >= kPerJobHistories * static_cast<uint64_t>(n_jobs);
    if (b->perJob) {
        b->hostJobs = J;
        for (int j = 0; j < n_jobs; ++j)
            b->jobShapes.push_back(chooseShape(worlds[j], opts[j], kernelTracking(J[j])));
        DXMCG_CUDA(b->jobCounters.alloc(n_jobs));
        DXMCG_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
        for (int k = 0; k < kBatchStreams; ++k) {
            DXMCG_CUDA(cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking));
            DXMCG_CUDA(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
        }
    }
    *out = b.release();
    return DXMCG_OK;
}

DXMCG_API int dxmcg_batch_info(const dxmcg_batch* b, int* n_jobs, uint64_t* job_histories, double* job_calibration)
{
    if (!b)
        return fail(DXMCG_ERR_ARGUMENT, "batch_info: null batch");
    const int n = static_cast<int>(b->worlds.size());
    if (n_jobs)
        *n_jobs = n;
    for (int j = 0; j < n; ++j) {
        if (job_histories)
            job_histories[j] = b->nHist[j];
        if (job_calibration)
            job_calibration[j] = b->calibration[j];
    }
    return DXMCG_OK;
}

DXMCG_API int dxmcg_batch_run(dxmcg_batch* b, dxmcg_stats* stats)
{
    const auto t0 = std::chrono::steady_clock::now();
    if (!b)
        return fail(DXMCG_ERR_ARGUMENT, "batch_run: null batch");
    DXMCG_CUDA(cudaSetDevice(b->device));
    const int nJobs = static_cast<int>(b->worlds.size());
    if (!b->exec) {
        DXMCG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        if (b->perJob) {
            // fork to the side streams, one launch per job round-robin, join
            e = cudaMemsetAsync(b->jobCounters.p, 0, nJobs * sizeof(DevCounters), b->stream);
            if (e == cudaSuccess)
                e = cudaEventRecord(b->fork, b->stream);
            for (int k = 0; k < kBatchStreams && e == cudaSuccess; ++k)
                e = cudaStreamWaitEvent(b->side[k], b->fork, 0);
            for (int j = 0; j < nJobs && e == cudaSuccess; ++j)
                e = launchTransport(b->hostJobs[j], b->nHist[j], b->jobCounters.p + j, b->jobShapes[j],
                    b->side[j % kBatchStreams]);
            for (int k = 0; k < kBatchStreams && e == cudaSuccess; ++k) {
                e = cudaEventRecord(b->join[k], b->side[k]);
                if (e == cudaSuccess)
                    e = cudaStreamWaitEvent(b->stream, b->join[k], 0);
            }
        } else {
            e = cudaMemsetAsync(b->counters.p, 0, sizeof(DevCounters), b->stream);
            if (e == cudaSuccess)
                e = launchTransportBatch(b->tracking, b->jobs.p, b->offsets.p, nJobs, b->total, b->counters.p,
                    b->shape, b->stream);
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess || ee != cudaSuccess) {
            if (g)
                cudaGraphDestroy(g);
            return cudaFail(e != cudaSuccess ? e : ee, "batch_run: graph capture");
        }
        b->graph = g;
        DXMCG_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    DXMCG_CUDA(cudaEventRecord(b->ev0, b->stream));
    DXMCG_CUDA(cudaGraphLaunch(b->exec, b->stream));
    DXMCG_CUDA(cudaEventRecord(b->ev1, b->stream));
    DevCounters c {};
    if (b->perJob) {
        std::vector<DevCounters> each(nJobs);
        DXMCG_CUDA(cudaMemcpyAsync(each.data(), b->jobCounters.p, nJobs * sizeof(DevCounters),
            cudaMemcpyDeviceToHost, b->stream));
        DXMCG_CUDA(cudaStreamSynchronize(b->stream));
        for (int j = 0; j < nJobs; ++j) {
            addCounters(c, each[j]);
            if (b->tracking == DXMCG_TRACK_WOODCOCK || b->tracking == kTrackWoodcockBox)
                noteStops(b->worlds[j], each[j]);
        }
    } else {
        DXMCG_CUDA(cudaMemcpyAsync(&c, b->counters.p, sizeof(c), cudaMemcpyDeviceToHost, b->stream));
        DXMCG_CUDA(cudaStreamSynchronize(b->stream));
    }
    float ms = 0.0f;
    DXMCG_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    for (size_t j = 0; j < b->worlds.size(); ++j)
        b->worlds[j]->historiesScored += static_cast<double>(b->nHist[j]);
    if (stats) {
        fillStats(c, stats);
        stats->n_cell_reads = b->gatherSkip ? c.visits - c.outer : 0;
        stats->kernel_ms = ms;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->dose_scale = kKeVToMilliGrayGram / b->worlds[0]->voxelVolume;
        stats->calibration = b->calibration[0];
        const bool wood = b->tracking == DXMCG_TRACK_WOODCOCK || b->tracking == kTrackWoodcockBox;
        stats->woodcock_steps = wood ? (b->perJob ? b->jobShapes[0].woodcock_steps : b->shape.woodcock_steps) : 0;
        stats->two_region = 0;
        if (b->perJob)
            for (const auto& hj : b->hostJobs)
                stats->two_region |= hj.boxOn;
        else
            stats->two_region = b->tracking == kTrackWoodcockBox ? 1 : 0;
    }
    return deviceErrors(c, "batch_run");
}

DXMCG_API void dxmcg_batch_destroy(dxmcg_batch* b) { delete b; }

DXMCG_API int dxmcg_autotune(dxmcg_world* w, const dxmcg_beam* beam, dxmcg_run_options* opts,
    uint64_t sample_histories, double* histories_per_second)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "autotune: world not built");
    if (!beam || !opts)
        return fail(DXMCG_ERR_ARGUMENT, "autotune: null beam or options");
    dxmcg_run_options o = *opts;
    if (o.tracking != DXMCG_TRACK_WOODCOCK && o.tracking != DXMCG_TRACK_SIDDON && o.tracking != DXMCG_TRACK_MACRO)
        return fail(DXMCG_ERR_ARGUMENT, "autotune: unknown tracking mode");
    o.normalize = 0; // trial runs need no calibration run
    DXMCG_CUDA(cudaSetDevice(w->device));
    DevJob J;
    uint64_t nHist = 0;
    double calibration = 1.0;
    int rc = prepareJob(w, *beam, o, J, nHist, calibration);
    if (rc != DXMCG_OK)
        return rc;
    if (nHist == 0)
        return fail(DXMCG_ERR_ARGUMENT, "autotune: the beam has no histories");
    // trials deposit into a scratch tally, never into the world's dose
    DeviceBuffer<Tally> scratch;
    DXMCG_CUDA(scratch.alloc(w->N));
    J.tally = scratch.p;
    const uint64_t n = std::min<uint64_t>(sample_histories > 0 ? sample_histories : (1ull << 24), nHist);
    const unsigned long long h0 = (nHist - n) / 2; // the middle of the beam's histories
    const unsigned long long h1 = h0 + n;

    auto trial = [&](const LaunchShape& shape, float& ms) -> int {
        DevCounters zero {};
        zero.next = h0;
        DXMCG_CUDA(cudaMemcpyAsync(w->counters.p, &zero, sizeof(zero), cudaMemcpyHostToDevice, w->stream));
        DXMCG_CUDA(cudaEventRecord(w->ev0, w->stream));
        const cudaError_t e = launchTransport(J, h1, w->counters.p, shape, w->stream);
        if (e != cudaSuccess)
            return cudaFail(e, "autotune: transport kernel launch");
        DXMCG_CUDA(cudaEventRecord(w->ev1, w->stream));
        DXMCG_CUDA(cudaEventSynchronize(w->ev1));
        DXMCG_CUDA(cudaEventElapsedTime(&ms, w->ev0, w->ev1));
        DevCounters c {};
        DXMCG_CUDA(cudaMemcpy(&c, w->counters.p, sizeof(c), cudaMemcpyDeviceToHost));
        return deviceErrors(c, "autotune");
    };

    static const int kBlocks[] = { 128, 256 };
    static const int kInteract[] = { 8, 12, 16, 24 };
    static const int kRefill[] = { 4, 8, 16 };
    static const int kWoodcock[] = { 4, 8, 12 };
    float warm = 0.0f;
    rc = trial(chooseShape(w, o, kernelTracking(J)), warm);
    if (rc != DXMCG_OK)
        return rc;
    float best = 0.0f;
    dxmcg_run_options bestOpt = o;
    for (int blk : kBlocks)
        for (int ib : kInteract)
            for (int rb : kRefill)
                for (int ws : kWoodcock) {
                    dxmcg_run_options t = o;
                    t.block_size = blk;
                    t.blocks_per_sm = 0;
                    t.interact_batch = ib;
                    t.refill_batch = rb;
                    t.woodcock_steps = o.tracking == DXMCG_TRACK_WOODCOCK ? ws : 0;
                    if (o.tracking != DXMCG_TRACK_WOODCOCK && ws != kWoodcock[0])
                        continue;
                    const LaunchShape shape = chooseShape(w, t, kernelTracking(J));
                    float m = 0.0f, m2 = 0.0f;
                    rc = trial(shape, m);
                    if (rc == DXMCG_OK)
                        rc = trial(shape, m2);
                    if (rc != DXMCG_OK)
                        return rc;
                    const float tmin = std::min(m, m2);
                    if (best == 0.0f || tmin < best) {
                        best = tmin;
                        bestOpt = t;
                    }
                }
    opts->block_size = bestOpt.block_size;
    opts->blocks_per_sm = 0;
    opts->interact_batch = bestOpt.interact_batch;
    opts->refill_batch = bestOpt.refill_batch;
    opts->woodcock_steps = bestOpt.woodcock_steps;
    if (histories_per_second)
        *histories_per_second = best > 0.0f ? static_cast<double>(n) / (best * 1e-3) : 0.0;
    return DXMCG_OK;
}

// ---------------------------------------------------------------- segmentation, dose table, readout

DXMCG_API int dxmcg_ct_segmentation_table(double kvp, double al_mm, double sn_mm, int n_materials,
    const dxmcg_material* materials, const double* densities, dxmcg_segmentation* out)
{
    if (!out || !materials || !densities || n_materials < 1 || n_materials > DXMCG_MAX_SEG_MATERIALS)
        return fail(DXMCG_ERR_ARGUMENT, "ct_segmentation_table: need 1..64 materials, densities and an output");
    if (!(kvp > 1.0))
        return fail(DXMCG_ERR_ARGUMENT, "ct_segmentation_table: bad tube voltage");
    for (int i = 0; i < n_materials; ++i)
        if (!validComposition(materials[i]) || !(densities[i] >= 0.0))
            return fail(DXMCG_ERR_ARGUMENT, "ct_segmentation_table: material " + std::to_string(i) + " is invalid");
    // Tube tube(kvp); setAlFiltration; setSnFiltration; getSpecter(energies, true)
    const int32_t fz[2] = { 13, 50 };
    const double fmm[2] = { std::max(0.0, al_mm), std::max(0.0, sn_mm) };
    const auto spec = tubeSpectrum(kvp, 12.0, 2, fz, fmm);
    const dxmcg_material water = waterMaterial(), air = dryAirMaterial();
    const double wd = 1.0, ad = 0.001205;
    *out = dxmcg_segmentation {};
    out->n_materials = n_materials;
    out->water_density = wd;
    out->air_density = ad;
    const size_t ne = spec.energy.size();
    std::vector<double> uw(ne), ua(ne);
    for (size_t k = 0; k < ne; ++k) {
        uw[k] = attenuation(water, 1, spec.energy[k]).sum();
        ua[k] = attenuation(air, 1, spec.energy[k]).sum();
        out->water_attenuation += spec.weight[k] * uw[k];
        out->air_attenuation += spec.weight[k] * ua[k];
    }
    for (int i = 0; i < n_materials; ++i) {
        double hu = 0.0, att = 0.0;
        for (size_t k = 0; k < ne; ++k) {
            const double um = attenuation(materials[i], 1, spec.energy[k]).sum();
            const double w = spec.weight[k];
            hu += w * (um * densities[i] - uw[k] * wd) / (uw[k] * wd - ua[k] * ad);
            att += w * um;
        }
        out->hu[i] = 1000.0 * hu;
        out->attenuation[i] = att;
    }
    for (int i = 0; i + 1 < n_materials; ++i)
        out->separator[i] = (out->hu[i] + out->hu[i + 1]) / 2;
    return DXMCG_OK;
}

DXMCG_API int dxmcg_ct_segment_device(const dxmcg_segmentation* table, const double* hu, uint64_t n,
    uint8_t* material, double* density, void* cuda_stream)
{
    SegTable t;
    int rc = toSegTable(table, t);
    if (rc != DXMCG_OK)
        return rc;
    if (n == 0)
        return DXMCG_OK;
    if (!hu || !material || !density)
        return fail(DXMCG_ERR_ARGUMENT, "ct_segment_device: null array");
    const double* lutD = nullptr;
    const uint8_t* lutM = nullptr;
    if ((rc = segLut(t, lutD, lutM)) != DXMCG_OK)
        return rc;
    const cudaError_t e
        = launchSegment(hu, n, t, lutD, lutM, material, density, static_cast<cudaStream_t>(cuda_stream));
    if (e != cudaSuccess)
        return cudaFail(e, "segmentation kernel launch");
    return DXMCG_OK;
}

DXMCG_API int dxmcg_ct_segment(const dxmcg_segmentation* table, const double* hu, uint64_t n, uint8_t* material,
    double* density)
{
    SegTable t;
    int rc = toSegTable(table, t);
    if (rc != DXMCG_OK)
        return rc;
    if (n == 0)
        return DXMCG_OK;
    if (!hu || !material || !density)
        return fail(DXMCG_ERR_ARGUMENT, "ct_segment: null array");
    if ((rc = currentDevice()) != DXMCG_OK)
        return rc;
    const double* lutD = nullptr;
    const uint8_t* lutM = nullptr;
    if ((rc = segLut(t, lutD, lutM)) != DXMCG_OK)
        return rc;
    const size_t chunk = std::min<uint64_t>(n, kStreamChunk);
    DeviceBuffer<double> dh, dd;
    DeviceBuffer<uint8_t> dm;
    DXMCG_CUDA(dh.alloc(chunk));
    DXMCG_CUDA(dd.alloc(chunk));
    DXMCG_CUDA(dm.alloc(chunk));
    for (uint64_t a = 0; a < n; a += chunk) {
        const size_t m = std::min<uint64_t>(chunk, n - a);
        DXMCG_CUDA(cudaMemcpy(dh.p, hu + a, m * sizeof(double), cudaMemcpyHostToDevice));
        const cudaError_t e = launchSegment(dh.p, m, t, lutD, lutM, dm.p, dd.p, nullptr);
        if (e != cudaSuccess)
            return cudaFail(e, "segmentation kernel launch");
        DXMCG_CUDA(cudaMemcpy(material + a, dm.p, m, cudaMemcpyDeviceToHost));
        DXMCG_CUDA(cudaMemcpy(density + a, dd.p, m * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return DXMCG_OK;
}

DXMCG_API int dxmcg_organ_dose_table_device(const uint8_t* organ, const double* dose, const double* density,
    uint64_t n, const double spacing_cm[3], int n_organs, dxmcg_organ_dose* out, void* cuda_stream)
{
    double V = 0;
    int rc = checkOrganArgs(spacing_cm, n_organs, out, V);
    if (rc != DXMCG_OK)
        return rc;
    if (n > 0 && (!organ || !dose || !density))
        return fail(DXMCG_ERR_ARGUMENT, "organ_dose_table_device: null array");
    const auto s = static_cast<cudaStream_t>(cuda_stream);
    OrganSums& sums = organSums();
    if ((rc = sums.alloc(s)) != DXMCG_OK)
        return rc;
    if (n > 0) {
        const cudaError_t e = launchOrganTable(organ, dose, density, n, V, n_organs, sums.cnt.p, sums.rho.p,
            sums.e.p, s);
        if (e != cudaSuccess)
            return cudaFail(e, "organ table kernel launch");
    }
    return sums.read(V, n_organs, out, s);
}

DXMCG_API int dxmcg_organ_dose_table(const uint8_t* organ, const double* dose, const double* density, uint64_t n,
    const double spacing_cm[3], int n_organs, dxmcg_organ_dose* out)
{
    double V = 0;
    int rc = checkOrganArgs(spacing_cm, n_organs, out, V);
    if (rc != DXMCG_OK)
        return rc;
    if (n > 0 && (!organ || !dose || !density))
        return fail(DXMCG_ERR_ARGUMENT, "organ_dose_table: null array");
    if ((rc = currentDevice()) != DXMCG_OK)
        return rc;
    OrganSums& sums = organSums();
    if ((rc = sums.alloc(nullptr)) != DXMCG_OK)
        return rc;
    const size_t chunk = std::max<uint64_t>(1, std::min<uint64_t>(n, kStreamChunk));
    DeviceBuffer<uint8_t> dor;
    DeviceBuffer<double> dd, dr;
    DXMCG_CUDA(dor.alloc(chunk));
    DXMCG_CUDA(dd.alloc(chunk));
    DXMCG_CUDA(dr.alloc(chunk));
    for (uint64_t a = 0; a < n; a += chunk) {
        const size_t m = std::min<uint64_t>(chunk, n - a);
        DXMCG_CUDA(cudaMemcpy(dor.p, organ + a, m, cudaMemcpyHostToDevice));
        DXMCG_CUDA(cudaMemcpy(dd.p, dose + a, m * sizeof(double), cudaMemcpyHostToDevice));
        DXMCG_CUDA(cudaMemcpy(dr.p, density + a, m * sizeof(double), cudaMemcpyHostToDevice));
        const cudaError_t e = launchOrganTable(dor.p, dd.p, dr.p, m, V, n_organs, sums.cnt.p, sums.rho.p, sums.e.p,
            nullptr);
        if (e != cudaSuccess)
            return cudaFail(e, "organ table kernel launch");
    }
    return sums.read(V, n_organs, out, nullptr);
}

DXMCG_API int dxmcg_world_organ_dose(dxmcg_world* w, const uint8_t* organ, int n_organs, int delete_air_dose,
    dxmcg_organ_dose* out)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "world_organ_dose: world not built");
    double V = 0;
    int rc = checkOrganArgs(w->spacing, n_organs, out, V);
    if (rc != DXMCG_OK)
        return rc;
    if (!organ)
        return fail(DXMCG_ERR_ARGUMENT, "world_organ_dose: null organ array");
    DXMCG_CUDA(cudaSetDevice(w->device));
    OrganSums& sums = organSums();
    if ((rc = sums.alloc(w->stream)) != DXMCG_OK)
        return rc;
    DeviceBuffer<uint8_t> dor;
    DXMCG_CUDA(dor.alloc(w->N));
    DXMCG_CUDA(cudaMemcpyAsync(dor.p, organ, w->N, cudaMemcpyHostToDevice, w->stream));
    const cudaError_t e = launchWorldOrganTable(dor.p, w->tally.p, w->vox.p, w->N, kKeVToMilliGrayGram / V,
        delete_air_dose ? 1 : 0, V, n_organs, sums.cnt.p, sums.rho.p, sums.e.p, w->stream);
    if (e != cudaSuccess)
        return cudaFail(e, "world organ table kernel launch");
    return sums.read(V, n_organs, out, w->stream);
}

DXMCG_API int dxmcg_world_read_dose_postprocessed(dxmcg_world* w, int delete_air_dose, double* dose,
    double* variance, double* count, int* micro_gray)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "world_read_dose_postprocessed: world not built");
    DXMCG_CUDA(cudaSetDevice(w->device));
    DeviceBuffer<double> d, v, c;
    DeviceBuffer<unsigned long long> mx;
    DeviceBuffer<int> micro;
    if (dose)
        DXMCG_CUDA(d.alloc(w->N));
    if (variance)
        DXMCG_CUDA(v.alloc(w->N));
    if (count)
        DXMCG_CUDA(c.alloc(w->N));
    DXMCG_CUDA(mx.alloc(1));
    DXMCG_CUDA(micro.alloc(1));
    const cudaError_t e = launchDosePostprocess(w->tally.p, w->vox.p, w->N, kKeVToMilliGrayGram / w->voxelVolume,
        w->historiesScored, delete_air_dose ? 1 : 0, mx.p, dose ? d.p : nullptr, variance ? v.p : nullptr,
        count ? c.p : nullptr, micro.p, w->stream);
    if (e != cudaSuccess)
        return cudaFail(e, "dose post-processing launch");
    if (dose)
        DXMCG_CUDA(cudaMemcpyAsync(dose, d.p, w->N * sizeof(double), cudaMemcpyDeviceToHost, w->stream));
    if (variance)
        DXMCG_CUDA(cudaMemcpyAsync(variance, v.p, w->N * sizeof(double), cudaMemcpyDeviceToHost, w->stream));
    if (count)
        DXMCG_CUDA(cudaMemcpyAsync(count, c.p, w->N * sizeof(double), cudaMemcpyDeviceToHost, w->stream));
    int mu = 0;
    DXMCG_CUDA(cudaMemcpyAsync(&mu, micro.p, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    if (micro_gray)
        *micro_gray = mu;
    return DXMCG_OK;
}

DXMCG_API int dxmcg_world_denoise(dxmcg_world* w, dxmcg_denoiser* d, double scale, double* dose_out,
    double* scale_used)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "world_denoise: world not built");
    if (!d)
        return fail(DXMCG_ERR_ARGUMENT, "world_denoise: null denoiser");
    DXMCG_CUDA(cudaSetDevice(w->device));
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    return nn::denoiseWorld(d, w->device, w->tally.p, w->vox.p, w->dims[0], w->dims[1], w->dims[2],
        kKeVToMilliGrayGram / w->voxelVolume, scale, dose_out, scale_used, w->stream);
}

DXMCG_API dxmcg_progress* dxmcg_progress_create(void) { return new dxmcg_progress(); }
DXMCG_API void dxmcg_progress_destroy(dxmcg_progress* p) { delete p; }
DXMCG_API void dxmcg_progress_get(const dxmcg_progress* p, uint64_t* done, uint64_t* total)
{
    if (!p)
        return;
    if (done)
        *done = p->done.load();
    if (total)
        *total = p->total.load();
}
DXMCG_API void dxmcg_progress_stop(dxmcg_progress* p)
{
    if (p)
        p->stop.store(1);
}
DXMCG_API void dxmcg_progress_reset(dxmcg_progress* p)
{
    if (!p)
        return;
    p->stop.store(0);
    p->done.store(0);
    p->total.store(1);
    p->setMessage("");
}
DXMCG_API int dxmcg_progress_continue(const dxmcg_progress* p) { return p ? !p->stop.load() : 1; }
DXMCG_API int dxmcg_progress_message(const dxmcg_progress* p, char* buf, int cap)
{
    if (!p || !buf || cap <= 0)
        return 0;
    auto* q = const_cast<dxmcg_progress*>(p);
    std::lock_guard<std::mutex> l(q->msgMutex);
    const int n = std::min<int>(cap - 1, static_cast<int>(q->message.size()));
    std::memcpy(buf, q->message.data(), n);
    buf[n] = 0;
    return n;
}

// ---------------------------------------------------------------- test hooks
DXMCG_API int dxmcg_siddon_trace(int n_rays, const float* origins, const float* directions, const int32_t dims[3],
    const float spacing[3], int cap, int64_t* voxel, float* length, int32_t* n_segments)
{
    if (n_rays < 0 || !origins || !directions || !dims || !spacing || cap < 1 || !voxel || !length || !n_segments)
        return fail(DXMCG_ERR_ARGUMENT, "siddon_trace: bad arguments");
    if (n_rays == 0)
        return DXMCG_OK;
    DeviceBuffer<float> o, d, l;
    DeviceBuffer<long long> v;
    DeviceBuffer<int> c;
    DXMCG_CUDA(o.alloc(3 * static_cast<size_t>(n_rays)));
    DXMCG_CUDA(d.alloc(3 * static_cast<size_t>(n_rays)));
    DXMCG_CUDA(v.alloc(static_cast<size_t>(n_rays) * cap));
    DXMCG_CUDA(l.alloc(static_cast<size_t>(n_rays) * cap));
    DXMCG_CUDA(c.alloc(n_rays));
    DXMCG_CUDA(cudaMemcpy(o.p, origins, 3 * sizeof(float) * n_rays, cudaMemcpyHostToDevice));
    DXMCG_CUDA(cudaMemcpy(d.p, directions, 3 * sizeof(float) * n_rays, cudaMemcpyHostToDevice));
    cudaError_t e = launchSiddon(n_rays, o.p, d.p, dims[0], dims[1], dims[2], spacing[0], spacing[1], spacing[2], cap,
        v.p, l.p, c.p, nullptr);
    if (e != cudaSuccess)
        return cudaFail(e, "siddon kernel");
    DXMCG_CUDA(cudaMemcpy(voxel, v.p, sizeof(long long) * n_rays * static_cast<size_t>(cap), cudaMemcpyDeviceToHost));
    DXMCG_CUDA(cudaMemcpy(length, l.p, sizeof(float) * n_rays * static_cast<size_t>(cap), cudaMemcpyDeviceToHost));
    DXMCG_CUDA(cudaMemcpy(n_segments, c.p, sizeof(int) * n_rays, cudaMemcpyDeviceToHost));
    return DXMCG_OK;
}

DXMCG_API int dxmcg_history_stream(uint64_t seed, uint32_t stream, uint64_t h0, int n_hist, int n_draws,
    uint32_t* out)
{
    if (n_hist < 0 || n_draws < 0 || !out)
        return fail(DXMCG_ERR_ARGUMENT, "history_stream: bad arguments");
    const size_t n = static_cast<size_t>(n_hist) * n_draws;
    if (n == 0)
        return DXMCG_OK;
    DeviceBuffer<uint32_t> o;
    DXMCG_CUDA(o.alloc(n));
    cudaError_t e = launchHistoryStream(streamKey(seed, stream), h0, n_hist, n_draws, o.p, nullptr);
    if (e != cudaSuccess)
        return cudaFail(e, "stream kernel");
    DXMCG_CUDA(cudaMemcpy(out, o.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return DXMCG_OK;
}

static int samplerCommon(int n, const double* energies, const dxmcg_material* m, const double* uniforms, int stride,
    DeviceBuffer<float>& E, DeviceBuffer<float>& U, DeviceBuffer<DevMaterial>& M)
{
    if (n < 0 || !energies || !m || !uniforms || stride < 1 || !validComposition(*m))
        return fail(DXMCG_ERR_ARGUMENT, "sampler: bad arguments");
    std::vector<float> e(n), u(static_cast<size_t>(n) * stride);
    for (int i = 0; i < n; ++i)
        e[i] = static_cast<float>(energies[i]);
    for (size_t i = 0; i < u.size(); ++i)
        u[i] = static_cast<float>(uniforms[i]);
    const DevMaterial dm = toDevMaterial(*m);
    DXMCG_CUDA(E.alloc(std::max(n, 1)));
    DXMCG_CUDA(U.alloc(std::max<size_t>(u.size(), 1)));
    DXMCG_CUDA(M.alloc(1));
    DXMCG_CUDA(cudaMemcpy(E.p, e.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    DXMCG_CUDA(cudaMemcpy(U.p, u.data(), sizeof(float) * u.size(), cudaMemcpyHostToDevice));
    DXMCG_CUDA(cudaMemcpy(M.p, &dm, sizeof(dm), cudaMemcpyHostToDevice));
    return DXMCG_OK;
}

DXMCG_API int dxmcg_sample_compton(int n, const double* energies, const dxmcg_material* m, int correction,
    const double* uniforms, int u_stride, double* e_out, double* cos_out, int32_t* used)
{
    if (!e_out || !cos_out || !used)
        return fail(DXMCG_ERR_ARGUMENT, "sample_compton: null output");
    DeviceBuffer<float> E, U, eo, co;
    DeviceBuffer<DevMaterial> M;
    DeviceBuffer<int> us;
    int rc = samplerCommon(n, energies, m, uniforms, u_stride, E, U, M);
    if (rc != DXMCG_OK || n == 0)
        return rc;
    DXMCG_CUDA(eo.alloc(n));
    DXMCG_CUDA(co.alloc(n));
    DXMCG_CUDA(us.alloc(n));
    std::vector<float> ctabHost(static_cast<size_t>(kNE) * kCTabK);
    buildComptonAngleTables(m, 1, correction, ctabHost.data());
    DeviceBuffer<float> ctab;
    DXMCG_CUDA(ctab.alloc(ctabHost.size()));
    DXMCG_CUDA(cudaMemcpy(ctab.p, ctabHost.data(), sizeof(float) * ctabHost.size(), cudaMemcpyHostToDevice));
    cudaError_t e = launchSampleCompton(n, E.p, M.p, ctab.p, correction, U.p, u_stride, eo.p, co.p, us.p, nullptr);
    if (e != cudaSuccess)
        return cudaFail(e, "compton kernel");
    std::vector<float> a(n), b(n);
    DXMCG_CUDA(cudaMemcpy(a.data(), eo.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
    DXMCG_CUDA(cudaMemcpy(b.data(), co.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
    DXMCG_CUDA(cudaMemcpy(used, us.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) {
        e_out[i] = a[i];
        cos_out[i] = b[i];
    }
    return DXMCG_OK;
}

DXMCG_API int dxmcg_sample_photoelectric(int n, const double* energies, const dxmcg_material* m,
    const double* uniforms, int u_stride, double* e_out, double* dz_out, int32_t* used)
{
    if (!e_out || !dz_out || !used)
        return fail(DXMCG_ERR_ARGUMENT, "sample_photoelectric: null output");
    DeviceBuffer<float> E, U, eo, dz;
    DeviceBuffer<DevMaterial> M;
    DeviceBuffer<int> us;
    int rc = samplerCommon(n, energies, m, uniforms, u_stride, E, U, M);
    if (rc != DXMCG_OK || n == 0)
        return rc;
    DXMCG_CUDA(eo.alloc(n));
    DXMCG_CUDA(dz.alloc(n));
    DXMCG_CUDA(us.alloc(n));
    cudaError_t e = launchSamplePhoto(n, E.p, M.p, U.p, u_stride, eo.p, dz.p, us.p, nullptr);
    if (e != cudaSuccess)
        return cudaFail(e, "photoelectric kernel");
    std::vector<float> a(n), b(n);
    DXMCG_CUDA(cudaMemcpy(a.data(), eo.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
    DXMCG_CUDA(cudaMemcpy(b.data(), dz.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
    DXMCG_CUDA(cudaMemcpy(used, us.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) {
        e_out[i] = a[i];
        dz_out[i] = b[i];
    }
    return DXMCG_OK;
}

DXMCG_API int dxmcg_sample_rayleigh(int n, const double* energies, const dxmcg_material* m, const double* uniforms,
    int u_stride, double* cos_out, int32_t* used)
{
    if (!cos_out || !used)
        return fail(DXMCG_ERR_ARGUMENT, "sample_rayleigh: null output");
    DeviceBuffer<float> E, U, co;
    DeviceBuffer<DevMaterial> M;
    DeviceBuffer<int> us;
    int rc = samplerCommon(n, energies, m, uniforms, u_stride, E, U, M);
    if (rc != DXMCG_OK || n == 0)
        return rc;
    DXMCG_CUDA(co.alloc(n));
    DXMCG_CUDA(us.alloc(n));
    std::vector<float> rtabHost(static_cast<size_t>(kNE) * kCTabK);
    buildRayleighAngleTables(m, 1, rtabHost.data());
    DeviceBuffer<float> rtab;
    DXMCG_CUDA(rtab.alloc(rtabHost.size()));
    DXMCG_CUDA(cudaMemcpy(rtab.p, rtabHost.data(), sizeof(float) * rtabHost.size(), cudaMemcpyHostToDevice));
    cudaError_t e = launchSampleRayleigh(n, E.p, M.p, rtab.p, U.p, u_stride, co.p, us.p, nullptr);
    if (e != cudaSuccess)
        return cudaFail(e, "rayleigh kernel");
    std::vector<float> b(n);
    DXMCG_CUDA(cudaMemcpy(b.data(), co.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
    DXMCG_CUDA(cudaMemcpy(used, us.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i)
        cos_out[i] = b[i];
    return DXMCG_OK;
}

DXMCG_API int dxmcg_umma_probe(int N, const uint16_t* a, const uint16_t* b0, const uint16_t* b1, float* d0,
    float* d1)
{
    if ((N != 16 && N != 32) || !a || !b0 || !b1 || !d0 || !d1)
        return fail(DXMCG_ERR_ARGUMENT, "umma_probe: N must be 16 or 32, all arrays given");
    DeviceBuffer<uint16_t> A, B0, B1;
    DeviceBuffer<float> D0, D1;
    DeviceBuffer<unsigned> st;
    DXMCG_CUDA(A.alloc(128 * 16));
    DXMCG_CUDA(B0.alloc(128 * 16));
    DXMCG_CUDA(B1.alloc(128 * 16));
    DXMCG_CUDA(D0.alloc(128 * N));
    DXMCG_CUDA(D1.alloc(128 * N));
    DXMCG_CUDA(st.alloc(1));
    DXMCG_CUDA(cudaMemset(B0.p, 0, 128 * 16 * sizeof(uint16_t)));
    DXMCG_CUDA(cudaMemset(B1.p, 0, 128 * 16 * sizeof(uint16_t)));
    DXMCG_CUDA(cudaMemset(st.p, 0, sizeof(unsigned)));
    DXMCG_CUDA(cudaMemcpy(A.p, a, 128 * 16 * sizeof(uint16_t), cudaMemcpyHostToDevice));
    DXMCG_CUDA(cudaMemcpy(B0.p, b0, N * 16 * sizeof(uint16_t), cudaMemcpyHostToDevice));
    DXMCG_CUDA(cudaMemcpy(B1.p, b1, N * 16 * sizeof(uint16_t), cudaMemcpyHostToDevice));
    cudaError_t e = launchUmmaProbe(A.p, B0.p, B1.p, N, D0.p, D1.p, st.p, nullptr);
    if (e != cudaSuccess)
        return cudaFail(e, "umma probe");
    unsigned status = 0;
    DXMCG_CUDA(cudaMemcpy(d0, D0.p, 128 * N * sizeof(float), cudaMemcpyDeviceToHost));
    DXMCG_CUDA(cudaMemcpy(d1, D1.p, 128 * N * sizeof(float), cudaMemcpyDeviceToHost));
    DXMCG_CUDA(cudaMemcpy(&status, st.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (status)
        return fail(DXMCG_ERR_DEVICE, "umma probe: the tensor-core commit was not seen in time");
    return DXMCG_OK;
}

DXMCG_API int dxmcg_sample_source(dxmcg_world* w, const dxmcg_beam* beam, const dxmcg_run_options* opts, int n,
    double* out8)
{
    if (!w || !w->built)
        return fail(DXMCG_ERR_STATE, "sample_source: world not built");
    if (!beam || n < 0 || !out8)
        return fail(DXMCG_ERR_ARGUMENT, "sample_source: bad arguments");
    dxmcg_run_options o {};
    o.seed = 1;
    if (opts)
        o = *opts;
    DXMCG_CUDA(cudaSetDevice(w->device));
    DevJob J;
    uint64_t nHist = 0;
    double calibration = 1.0;
    int rc = prepareJob(w, *beam, o, J, nHist, calibration);
    if (rc != DXMCG_OK)
        return rc;
    DXMCG_CUDA(cudaSetDevice(w->device));
    if (o.hist_begin + static_cast<uint64_t>(n) > nHist)
        return fail(DXMCG_ERR_ARGUMENT, "sample_source: history range beyond the beam");
    if (n == 0)
        return DXMCG_OK;
    DeviceBuffer<float> out;
    DXMCG_CUDA(out.alloc(8 * static_cast<size_t>(n)));
    cudaError_t e = launchSampleSource(J, o.hist_begin, n, out.p, w->stream);
    if (e != cudaSuccess)
        return cudaFail(e, "source kernel");
    std::vector<float> h(8 * static_cast<size_t>(n));
    DXMCG_CUDA(cudaMemcpyAsync(h.data(), out.p, h.size() * sizeof(float), cudaMemcpyDeviceToHost, w->stream));
    DXMCG_CUDA(cudaStreamSynchronize(w->stream));
    for (size_t i = 0; i < h.size(); ++i)
        out8[i] = h[i];
    return DXMCG_OK;
}

} // extern "C"
