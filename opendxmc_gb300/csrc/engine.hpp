// engine.hpp -- device data layout and kernel launchers shared by the host
// library (capi.cpp) and the kernels (transport.cu).
//
// HBM layout of one world (N = nx*ny*nz voxels):
//   vox    uint32[N]   density with the low 8 mantissa bits replaced by the
//                      material index (one 4-byte gather per voxel visit;
//                      density keeps 16 significant bits, |rel. rounding| <= 2^-16)
//   tally  Tally[N]    {energy, energy^2, events} in one 32-byte sector
//   tot    float[M][NE]        total mass attenuation per material (cm^2/g)
//   xs     float4[M][NE]       (photo, incoherent, coherent, total)
//   maj    float[NE]           majorant mu_max(E) over the grid (1/cm)
//   mats   DevMaterial[M]      per-element sampling data
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dxmcg.h"

namespace dxmcg {

constexpr int kMaxSpectrum = 512;
constexpr int kMaxBowtie = 64;
constexpr int kTableNE = DXMCG_NE;
constexpr uint32_t kMaxStepsPerHistory = 1000000;
constexpr int kMaxRejections = 100000;
// Compton and Rayleigh angles: per material and table energy E_i, 1 - cos theta at the
// cumulative probabilities u_j = (1 - cos(pi j / (kCTabK - 1)))/2 of the Klein-Nishina x
// S(x) / Z distribution (S = 1 at correction 0), or of the Rayleigh distribution
// (1 + cos^2)/2 F^2(x), j = 0 .. kCTabK - 1: 2 at j = 0, 0 at the last.  The u grid is
// densest at both ends: the narrow forward peak and the long backward tail.
constexpr int kCTabK = 256;

struct DevMaterial {
    int n;
    float Zsum;
    float nZ[DXMCG_MAX_ELEMENTS];
    float nZ2[DXMCG_MAX_ELEMENTS];
    float a[DXMCG_MAX_ELEMENTS];
    float ia[DXMCG_MAX_ELEMENTS]; // 1 / a
    // correction level 2: photoelectric element choice and K fluorescence
    float nZ4[DXMCG_MAX_ELEMENTS];
    float eK[DXMCG_MAX_ELEMENTS];
    float eL[DXMCG_MAX_ELEMENTS];
    float kAlpha[DXMCG_MAX_ELEMENTS];
    float omegaK[DXMCG_MAX_ELEMENTS];
    float invJumpK, invJumpL;
    // correction level 2: Compton shells of the material (all elements)
    int nShell;
    float shellElectrons[3 * DXMCG_MAX_ELEMENTS];
    float shellBinding[3 * DXMCG_MAX_ELEMENTS];
    float shellMomentum[3 * DXMCG_MAX_ELEMENTS];
};

struct alignas(16) DevExposure {
    float pos[3]; // grid-local cm
    float c0[3];
    float c1[3];
    float n[3];   // c0 x c1
    float half[2];
    float weight;
    int tube;
};

static_assert(sizeof(DevExposure) == 64, "the source sampler reads an exposure as four float4");

struct DevSpectrum {
    int n;
    float E[kMaxSpectrum];
    uint32_t thr[kMaxSpectrum];
    int32_t alias[kMaxSpectrum];
};

// One bowtie profile per tube (tube 1: dual-energy tube B); n[t] = 0 leaves that
// tube's weights at 1 (and inv_norm[t] = 1).  seg[t][c] is a segment near the angles
// of cell c of kBowtieCells equal cells over [0, ang[t][n-1]] (cellScale = cells per
// radian): the lookup starts there instead of a binary search.
constexpr int kBowtieCells = 256;
struct DevBowtie {
    int n[2];
    float ang[2][kMaxBowtie];
    float w[2][kMaxBowtie];
    float inv_norm[2];
    float cellScale[2];
    uint8_t seg[2][kBowtieCells];
};

struct alignas(32) Tally {
    double e;
    double e2;
    unsigned long long n;
    unsigned long long pad;
};

struct DevJob {
    // world
    const uint32_t* vox;
    const float* dens;   // unpacked voxel arrays (the allocation-free entry point)
    const uint8_t* mat;
    int nx, ny, nz;
    float sp[3];
    float isp[3];
    float L[3];
    float Lin[3]; // largest float strictly below L
    const float* tot;
    const float4* xs;
    const float* maj;
    const DevMaterial* mats;
    const float* rtab; // [n_mats][kTableNE][kCTabK] Rayleigh 1 - cos theta quantiles
    const float* ctab; // [n_mats][kTableNE][kCTabK] Compton 1 - cos theta quantiles
    int n_mats;
    int correction;
    Tally* tally;
    // macro cells (MACRO tracking): scale s_c per cell of mb^3 voxels
    const float* mscale;
    int mc[3];
    int mb;
    float cellL[3]; // cell edge in cm
    // source
    const DevExposure* exps;
    int n_exp;
    unsigned long long ppe;
    const DevSpectrum* spec; // [2]
    const DevBowtie* bowtie; // nullptr: no bowtie on either tube
    int beam_type;
    float pencil_energy;
    unsigned long long key; // streamKey(seed, stream word) of the run
    int tracking;
    uint32_t maxSteps; // per-history step limit (kErrStepLimit beyond it)
    // Woodcock gather skip: per cell of kCellEdge^3 voxels an upper bound b_c of
    // rho mu_m(E) / mu_max(E) over the cell's voxels and all energies (+inf where the
    // cell holds a transparent voxel); nullptr: off.  cb[0], cb[1]: cells along x, y.
    const float* cbound;
    int cb[2];
    // Two-region Woodcock: every voxel outside the box of voxels whose material is not
    // 0 (nor transparent) holds material 0, so a flight that starts outside the box
    // steps against majOut(E) >= rho mu_0(E) of those voxels until it reaches the box,
    // and against maj(E) from there on.  Box voxel indices b0 .. b0 + bn - 1; blo, bhi:
    // its faces in cm, widened by a margin (a flight may reach it early, never late).
    // boxOn 0: one region.
    int boxOn;
    int b0[3];
    unsigned bn[3];
    float blo[3], bhi[3];
    const float* majOut;
};

constexpr int kCellShift = 3; // gather-skip cells of 8 x 8 x 8 voxels
constexpr int kCellEdge = 1 << kCellShift;

struct DevCounters {
    unsigned long long next; // work-queue head (history index)
    unsigned long long histories, missed, visits, photo, compton, rayleigh, cutoff, errors, interacted, crossings,
        fluorescence;
    double e_source, e_escaped, e_deposited;
    unsigned int error_flags;
    unsigned long long skipped; // Woodcock tentative collisions settled by the cell bound alone
    unsigned long long outer;   // two-region Woodcock: tentative collisions outside the box (no cell bound)
};

enum ErrorFlag : unsigned {
    kErrStepLimit = 1u,
    kErrRejectLimit = 2u,
    kErrBadDensity = 4u,
    kErrBadMaterial = 8u,
};

struct LaunchShape {
    int grid = 0;
    int block = 256;
    int refill_batch = 0;   // dead lanes a warp gathers before starting new histories (0: default)
    int interact_batch = 0; // parked lanes a warp gathers before running scatterings (0: default)
    int woodcock_steps = 0; // Woodcock steps per lane and step phase (0: default)
};

// Per-history random streams.  splitMix64 is the output function of SplitMix64
// (Steele, Lea & Flood 2014), a bijection of the 64-bit integers that passes BigCrush on
// a counter.  streamKey mixes a run's (seed, stream word) into the key its histories'
// streams start from: distinct seeds with one stream word, or one seed with distinct
// stream words, give distinct keys.
__host__ __device__ __forceinline__ unsigned long long splitMix64(unsigned long long z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
constexpr unsigned long long kGolden64 = 0x9E3779B97F4A7C15ull;
__host__ __device__ __forceinline__ unsigned long long streamKey(unsigned long long seed, uint32_t stream)
{
    return splitMix64(seed ^ splitMix64(static_cast<unsigned long long>(stream) + kGolden64));
}

// Kernel instances of the transport are chosen by "kernel tracking": the public
// DXMCG_TRACK_* modes, and kTrackWoodcockBox, Woodcock tracking with two regions,
// for jobs whose world has a two-region box (DevJob::boxOn).
constexpr int kTrackWoodcockBox = 3;
inline int kernelTracking(const DevJob& J)
{
    return J.tracking == DXMCG_TRACK_WOODCOCK && J.boxOn ? kTrackWoodcockBox : J.tracking;
}

// kernels (transport.cu)
cudaError_t launchPack(const double* dens64, const float* dens32, const uint8_t* mat, uint32_t* vox, size_t n,
    int n_mats, unsigned* rho_max_bits, unsigned* err, cudaStream_t s);
cudaError_t launchTransport(const DevJob& job, unsigned long long h_end, DevCounters* ctr, LaunchShape shape,
    cudaStream_t s);
// per-macro-cell majorant scale: max over the cell's voxels of rho * ratio[m]
cudaError_t launchMacroScale(const uint32_t* vox, int nx, int ny, int nz, int mb, int mcx, int mcy,
    const float* ratio, unsigned* scaleBits, cudaStream_t s);
// gather-skip bounds: per cell of kCellEdge^3 voxels (cells x fastest, ncx x ncy x ncz)
// max over its voxels of rho * ratio[m] times (1 + 2^-12), +inf if one is transparent
// bounding box of the voxels whose material is neither 0 nor transparent:
// box = {min x, min y, min z, max x, max y, max z}, initialised by the caller to
// {INT_MAX x3, -1 x3} (max x = -1 after the launch: no such voxel)
cudaError_t launchMaterialBox(const uint32_t* vox, int nx, int ny, int nz, int* box, cudaStream_t s);
cudaError_t launchMaterialBox(const uint8_t* mat, int nx, int ny, int nz, int* box, cudaStream_t s);
cudaError_t launchCellBound(const uint32_t* vox, int nx, int ny, int nz, int ncx, int ncy, int ncz, const float* ratio,
    float* bound, cudaStream_t s);
cudaError_t launchFinalize(const Tally* tally, const uint32_t* vox, size_t n, double energy_to_dose,
    double n_histories, double* dose, double* var, unsigned long long* count, cudaStream_t s);
cudaError_t launchSiddon(int n_rays, const float* o, const float* d, int nx, int ny, int nz, float sx, float sy,
    float sz, int cap, long long* idx, float* len, int* cnt, cudaStream_t s);
cudaError_t launchSampleCompton(int n, const float* E, const DevMaterial* m, const float* ctab, int correction,
    const float* u, int stride, float* e_out, float* cos_out, int* used, cudaStream_t s);
cudaError_t launchSamplePhoto(int n, const float* E, const DevMaterial* m, const float* u, int stride, float* e_out,
    float* dz_out, int* used, cudaStream_t s);
// tcgen05 interface self-test (conv_tc.cu): D0 = A (B0 + B1)^T, D1 = A B1^T, A 128 x 16,
// B N x 16 (N = 16 or 32) bf16 row-major, D FP32 [128][N]; *status |= 1 on a timed-out wait
cudaError_t launchUmmaProbe(const uint16_t* A, const uint16_t* B0, const uint16_t* B1, int N, float* D0, float* D1,
    unsigned* status, cudaStream_t s);
cudaError_t launchSampleRayleigh(int n, const float* E, const DevMaterial* m, const float* rtab, const float* u,
    int stride, float* cos_out, int* used, cudaStream_t s);
cudaError_t launchSampleSource(const DevJob& job, unsigned long long h0, int n, float* out8, cudaStream_t s);
cudaError_t launchHistoryStream(unsigned long long key, unsigned long long h0, int n_hist, int n_draws,
    uint32_t* out, cudaStream_t s);
int transportRegistersPerThread(int tracking);
int transportMaxBlocksPerSM(int block, int tracking);
// the same kernel reading caller-owned float density / uint8 material arrays
cudaError_t launchTransportUnpacked(const DevJob& job, unsigned long long h_end, DevCounters* ctr,
    LaunchShape shape, cudaStream_t s);
int transportMaxBlocksPerSMUnpacked(int block, int tracking);
// one persistent launch over several jobs (device descriptors `jobs`, packed worlds):
// offsets[j] is job j's first history in the shared queue, offsets[nJobs] == h_end
cudaError_t launchTransportBatch(int tracking, const DevJob* jobs, const unsigned long long* offsets, int nJobs,
    unsigned long long h_end, DevCounters* ctr, LaunchShape shape, cudaStream_t s);
int transportMaxBlocksPerSMBatch(int block, int tracking);

// per-voxel passes around the transport (pipelines.cu)
constexpr int kMaxSegMaterials = 64;
struct SegTable {
    int nSep = 0;       // number of separators (materials - 1)
    double slope = 0;   // w_att * w_dens - a_att * a_dens
    double offset = 0;  // w_att * w_dens
    double sep[kMaxSegMaterials - 1] {}; // HU midpoints between consecutive materials
    double att[kMaxSegMaterials] {};     // spectrum-weighted mass attenuation per material
};
// lookup table for integer CT numbers [kSegLutMin, kSegLutMin + kSegLutSize): density
// and material of each, computed on the host with the kernel's FP64 operations
constexpr int kSegLutMin = -1024;
constexpr int kSegLutSize = 4096;
void segmentHost(double h, const SegTable& t, uint8_t& m, double& d);
cudaError_t launchSegment(const double* hu, size_t n, const SegTable& t, const double* lutD, const uint8_t* lutM,
    uint8_t* mat, double* dens, cudaStream_t s);
cudaError_t launchOrganTable(const uint8_t* organ, const double* dose, const double* density, size_t n,
    double voxel_volume, int n_organs, unsigned long long* cnt, double* sum_rho, double* sum_e, cudaStream_t s);
cudaError_t launchWorldOrganTable(const uint8_t* organ, const Tally* tally, const uint32_t* vox, size_t n,
    double energy_to_dose, int air_mask, double voxel_volume, int n_organs, unsigned long long* cnt,
    double* sum_rho, double* sum_e, cudaStream_t s);
cudaError_t launchDosePostprocess(const Tally* tally, const uint32_t* vox, size_t n, double energy_to_dose,
    double n_histories, int air_mask, unsigned long long* max_bits, double* dose, double* var, double* count,
    int* micro, cudaStream_t s);

// host helpers (geometry.cpp)
int expandExposures(const dxmcg_beam& b, std::vector<dxmcg_exposure>& out);
// sets the calling thread's dxmcg_last_error() text and returns code (capi.cpp)
int reportError(int code, const std::string& msg);
// dose calibration (calibration.cpp): DAP per history of the beam's spectrum, and the
// factor F applied to every history weight when opts.normalize is set
double dapPerHistory(const dxmcg_beam& b);
// air kerma (mGy) of one pencil-beam history per cm2: E (mu_tr/rho)_air(E)
double airKermaPerHistory(const dxmcg_beam& b);
int calibrationFactor(const dxmcg_beam& b, int correction, const dxmcg_run_options& o, uint64_t nHist,
    bool allowPhantom, double& F, std::string& err);

} // namespace dxmcg
