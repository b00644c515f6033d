// transport.cu -- the persistent photon-transport kernel (sm_103a).
//
// Every lane owns one photon and is in one of five states: stepping, waiting for
// a Compton interaction, waiting for a Rayleigh interaction, waiting for the
// fluorescence of a photoelectric absorption (correction level 2), or dead.  Each
// loop iteration of a warp has three phases whose branches are warp-uniform:
//
//   refill    dead lanes start new histories (source sampling, entry into the
//             grid) once at least `refillBatch` lanes are dead, from a warp-private
//             pool of history indices that the warp takes from a global work-queue
//             head in chunks of kChunk (one atomic per chunk);
//   interact  lanes waiting for an interaction run it together once at least
//             `interactBatch` lanes wait (Compton: the angle from the material's
//             Klein-Nishina x S(x)/Z quantile table, and at level 2 the Doppler
//             energy of a bound electron; Rayleigh: element choice from the
//             material's share table and analytic inversion of F^2, rejection on
//             (1 + cos^2)/2; fluorescence: K-shell vacancy and yield);
//   step      stepping lanes take up to `woodcockSteps` Woodcock steps against the
//             majorant mu_max(E), stopping at a real collision or an escape (or, in
//             the regular-tracking variant, one free flight with exact Siddon path
//             lengths; with macro cells, one flight against the cell majorants); a
//             real collision picks its type at once: photoelectric absorption is
//             scored on the spot below level 2, the other events park the lane
//             until the next interact phase.
//
// Parking interactions and batching refills regroups the expensive, divergent
// work so that it runs with many lanes active instead of one or two.  A history
// draws its uniforms in a fixed order from its own stream, so its result does not
// depend on when, or in which lane, each phase runs.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "device.cuh"

namespace dxmcg {
namespace {
    using namespace dev;

    constexpr int kChunk = 256; // histories a warp takes from the queue at once

    // kPhoto: a photoelectric absorption waiting for its fluorescence (correction level 2)
    enum LaneState : int { kDead = 0, kStepping = 1, kCompton = 2, kRayleigh = 3, kPhoto = 4 };
    enum BlockCount : int {
        cHist,
        cMissed,
        cPhoto,
        cCompton,
        cRayleigh,
        cCutoff,
        cErrors,
        cInteracted,
        cFluorescence,
        cNum
    };

    __device__ __forceinline__ unsigned long long warpSum(unsigned long long v)
    {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(kFull, v, o);
        return v;
    }
    __device__ __forceinline__ double warpSum(double v)
    {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(kFull, v, o);
        return v;
    }

    // Kahan-compensated FP32 sum; value() returns it in FP64 once, at the end.
    struct KahanSum {
        float s = 0.0f, c = 0.0f;
        __device__ __forceinline__ void add(float x)
        {
            const float y = x - c;
            const float t = s + y;
            c = (t - s) - y;
            s = t;
        }
        __device__ __forceinline__ double value() const { return static_cast<double>(s) - static_cast<double>(c); }
    };

    // Per-thread sums of the source, escaped and deposited energy (K = 0, 1, 2), and
    // the warp's pool of history indices [next, end) with its exhausted flag, in
    // registers (LaneTotals<false>) or in shared memory (LaneTotals<true>; sums: value
    // sEnergy[2K][thread], compensation [2K + 1]).  They change a few times per history
    // or once per refill phase, so shared memory costs little where registers are short.
    constexpr int kSumSource = 0, kSumEscaped = 1, kSumDeposited = 2;
    __shared__ float sEnergy[6][256];
    __shared__ unsigned long long sPool[256 / 32][2];
    __shared__ int sExhausted[256 / 32];

    template <bool SHARED>
    struct LaneTotals;

    template <>
    struct LaneTotals<false> {
        KahanSum sum[3];
        unsigned long long next = 0, end = 0;
        bool done = false;
        __device__ __forceinline__ void init() { }
        template <int K>
        __device__ __forceinline__ void add(float x)
        {
            sum[K].add(x);
        }
        template <int K>
        __device__ __forceinline__ double value() const
        {
            return sum[K].value();
        }
        __device__ __forceinline__ bool exhausted() const { return done; }
        __device__ __forceinline__ void markExhausted() { done = true; }
        __device__ __forceinline__ void loadPool(unsigned long long& n, unsigned long long& e) const
        {
            n = next;
            e = end;
        }
        __device__ __forceinline__ void storePool(unsigned long long n, unsigned long long e)
        {
            next = n;
            end = e;
        }
    };

    template <>
    struct LaneTotals<true> {
        __device__ __forceinline__ void init()
        {
#pragma unroll
            for (int k = 0; k < 6; ++k)
                sEnergy[k][threadIdx.x] = 0.0f;
            if ((threadIdx.x & 31u) == 0) {
                sPool[threadIdx.x >> 5][0] = sPool[threadIdx.x >> 5][1] = 0ull;
                sExhausted[threadIdx.x >> 5] = 0;
            }
            __syncwarp();
        }
        template <int K>
        __device__ __forceinline__ void add(float x)
        {
            const float c = sEnergy[2 * K + 1][threadIdx.x], s0 = sEnergy[2 * K][threadIdx.x];
            const float y = x - c;
            const float t = s0 + y;
            sEnergy[2 * K + 1][threadIdx.x] = (t - s0) - y;
            sEnergy[2 * K][threadIdx.x] = t;
        }
        template <int K>
        __device__ __forceinline__ double value() const
        {
            return static_cast<double>(sEnergy[2 * K][threadIdx.x])
                - static_cast<double>(sEnergy[2 * K + 1][threadIdx.x]);
        }
        __device__ __forceinline__ bool exhausted() const { return sExhausted[threadIdx.x >> 5] != 0; }
        // warp-uniform: every lane calls it; one writes, the barrier publishes
        __device__ __forceinline__ void markExhausted()
        {
            __syncwarp();
            if ((threadIdx.x & 31u) == 0)
                sExhausted[threadIdx.x >> 5] = 1;
            __syncwarp();
        }
        __device__ __forceinline__ void loadPool(unsigned long long& n, unsigned long long& e) const
        {
            n = sPool[threadIdx.x >> 5][0];
            e = sPool[threadIdx.x >> 5][1];
        }
        __device__ __forceinline__ void storePool(unsigned long long n, unsigned long long e)
        {
            __syncwarp();
            if ((threadIdx.x & 31u) == 0) {
                sPool[threadIdx.x >> 5][0] = n;
                sPool[threadIdx.x >> 5][1] = e;
            }
            __syncwarp();
        }
    };

    // The photon's energy-grid position and the majorant its next flight steps
    // against.  A negative invMmax marks a flight outside the two-region box, against
    // majOut(E) = mmax = -1 / invMmax (no extra loop-carried register).
    struct EnergyCache {
        int ie;
        float fe, mmax, invMmax;
        __device__ __forceinline__ void set(const DevJob& J, float E)
        {
            gridPos(E, ie, fe);
            toInner(J);
        }
        __device__ __forceinline__ void toInner(const DevJob& J)
        {
            mmax = lerp1(J.maj, ie, fe);
            invMmax = 1.0f / mmax;
        }
        __device__ __forceinline__ void toOuter(const DevJob& J)
        {
            mmax = lerp1(J.majOut, ie, fe);
            invMmax = -1.0f / mmax;
        }
    };

    // Per-thread count of tentative collisions outside the two-region box (they read
    // their voxel without the cell bound); about one per history, so kept in shared
    // memory rather than in a register across the transport loop.
    __shared__ unsigned sOuterVisits[256];

    // Voxel (ix, iy, iz) lies outside the two-region box.
    __device__ __forceinline__ bool outsideBox(const DevJob& J, int ix, int iy, int iz)
    {
        return (static_cast<unsigned>(ix - J.b0[0]) >= J.bn[0]) | (static_cast<unsigned>(iy - J.b0[1]) >= J.bn[1])
            | (static_cast<unsigned>(iz - J.b0[2]) >= J.bn[2]);
    }

    // Distance along the flight to the widened box (FLT_MAX if the line misses it, 0
    // from inside it).  Approximate reciprocals: the margin of the box absorbs their
    // error, so the entry is never found late.
    __device__ __forceinline__ float boxEntry(const DevJob& J, const Photon& ph)
    {
        const float p[3] = { ph.px, ph.py, ph.pz };
        const float d[3] = { ph.dx, ph.dy, ph.dz };
        float tn = 0.0f, tf = FLT_MAX;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float inv = __fdividef(1.0f, d[a]);
            const float t1 = (J.blo[a] - p[a]) * inv, t2 = (J.bhi[a] - p[a]) * inv;
            tn = fmaxf(tn, fminf(t1, t2));
            tf = fminf(tf, fmaxf(t1, t2));
        }
        return tn <= tf ? tn : FLT_MAX;
    }

    // Density and material of voxel v: one 4-byte word in the packed layout, or two
    // loads from caller-owned arrays in the unpacked layout.
    template <bool PACKED>
    __device__ __forceinline__ float voxelAt(const DevJob& J, uint32_t v, int& m)
    {
        if (PACKED) {
            const uint32_t word = __ldg(J.vox + v);
            m = static_cast<int>(word & 0xffu);
            return __uint_as_float(word & 0xffffff00u);
        }
        m = static_cast<int>(__ldg(J.mat + v));
        return __ldg(J.dens + v);
    }

    // Woodcock step; returns true on a real collision in voxel v / material m.
    //
    // Gather skip (J.cbound set): the tentative collision is real when u mu_max(E) <
    // rho mu_m(E).  The cell's bound b_c satisfies rho mu_m(E) <= b_c mu_max(E) for each
    // of its voxels, with a margin larger than the FP32 roundings of both sides, so
    // u mu_max >= b_c mu_max settles the step as virtual without reading the voxel.
    // Otherwise the voxel is read and the usual test decides, on the same uniform: the
    // decisions, and so the histories, are those of the plain step.  Cells holding a
    // transparent voxel (b_c = +inf) take the plain step, which draws the uniform only
    // for a voxel that is not transparent.
    //
    // BOX (the two-region instance, for jobs with J.boxOn): a flight outside the box
    // steps against majOut; if the box comes first, the photon moves to it and steps
    // on against maj (the flight is memoryless), drawing no acceptance uniform.  A
    // flight against maj that ends outside the box decides its tentative collision as
    // usual (maj bounds every voxel); the flights after it step against majOut.  Every
    // decision keeps the tentative-collision rate at or above rho mu(E) on the path, so
    // the transport is that of plain Woodcock with fewer tentative collisions.  Outside
    // the box the cell bounds (relative to maj) are not used.
    template <bool PACKED, bool BOX>
    __device__ __forceinline__ bool woodcockStep(const DevJob& J, Photon& ph, Rng& rng, EnergyCache& ec,
        bool& escaped, uint32_t& v, int& m, unsigned& visits, unsigned& skipped)
    {
        const bool outer = BOX && ec.invMmax < 0.0f;
        // hardware log2: |error| <= 2^-21.4 near u = 1, where the step is < 1e-6 mean free paths
        const float s = fmaxf(-__logf(rng.u()), 0.0f) * (BOX ? fabsf(ec.invMmax) : ec.invMmax);
        if (BOX && outer) {
            const float te = boxEntry(J, ph);
            if (te < s) {
                ph.px = fmaf(te, ph.dx, ph.px);
                ph.py = fmaf(te, ph.dy, ph.py);
                ph.pz = fmaf(te, ph.dz, ph.pz);
                ec.toInner(J);
                return false;
            }
        }
        ph.px = fmaf(s, ph.dx, ph.px);
        ph.py = fmaf(s, ph.dy, ph.py);
        ph.pz = fmaf(s, ph.dz, ph.pz);
        // voxel indices by rounding down; outside the grid one of them is negative
        // (huge as unsigned) or >= its dimension (conversions saturate far away)
        const int ix = __float2int_rd(ph.px * J.isp[0]);
        const int iy = __float2int_rd(ph.py * J.isp[1]);
        const int iz = __float2int_rd(ph.pz * J.isp[2]);
        if ((static_cast<unsigned>(ix) >= static_cast<unsigned>(J.nx))
            | (static_cast<unsigned>(iy) >= static_cast<unsigned>(J.ny))
            | (static_cast<unsigned>(iz) >= static_cast<unsigned>(J.nz))) {
            escaped = true;
            return false;
        }
        ++visits;
        v = static_cast<uint32_t>(ix + J.nx * (iy + J.ny * iz));
        if (!BOX) {
            if (J.cbound) {
                const float b = __ldg(J.cbound
                    + ((ix >> kCellShift) + J.cb[0] * ((iy >> kCellShift) + J.cb[1] * (iz >> kCellShift))));
                if (b <= FLT_MAX) {
                    const float t = rng.u() * ec.mmax;
                    if (t >= b * ec.mmax) {
                        ++skipped;
                        return false;
                    }
                    const float rho = voxelAt<PACKED>(J, v, m);
                    return t < rho * lerp1(J.tot + m * kTableNE, ec.ie, ec.fe);
                }
            }
            const float rho = voxelAt<PACKED>(J, v, m);
            if (m == DXMCG_TRANSPARENT_MATERIAL)
                return false;
            const float mu = rho * lerp1(J.tot + m * kTableNE, ec.ie, ec.fe);
            return rng.u() * ec.mmax < mu;
        }
        if (outer)
            ++sOuterVisits[threadIdx.x];
        bool real = false, decided = false;
        if (J.cbound && !outer) {
            const float b = __ldg(J.cbound
                + ((ix >> kCellShift) + J.cb[0] * ((iy >> kCellShift) + J.cb[1] * (iz >> kCellShift))));
            if (b <= FLT_MAX) {
                decided = true;
                const float t = rng.u() * ec.mmax;
                if (t >= b * ec.mmax) {
                    ++skipped;
                } else {
                    const float rho = voxelAt<PACKED>(J, v, m);
                    real = t < rho * lerp1(J.tot + m * kTableNE, ec.ie, ec.fe);
                }
            }
        }
        if (!decided) {
            const float rho = voxelAt<PACKED>(J, v, m);
            if (m != DXMCG_TRANSPARENT_MATERIAL)
                real = rng.u() * ec.mmax < rho * lerp1(J.tot + m * kTableNE, ec.ie, ec.fe);
        }
        if (J.boxOn && !outer && outsideBox(J, ix, iy, iz))
            ec.toOuter(J);
        return real;
    }

    // One free flight with exact voxel path lengths; true on a collision.
    template <bool PACKED>
    __device__ __forceinline__ bool siddonFlight(const DevJob& J, Photon& ph, Rng& rng, const EnergyCache& ec,
        bool& escaped, uint32_t& v, int& m, unsigned& visits)
    {
        const float tau = -logf(rng.u());
        const float o[3] = { ph.px, ph.py, ph.pz };
        const float d[3] = { ph.dx, ph.dy, ph.dz };
        const int dims[3] = { J.nx, J.ny, J.nz };
        Siddon sd;
        float thit = 0.0f;
        bool hit = false;
        if (sd.begin(o, d, dims, J.sp)) {
            float acc = 0.0f;
            while (!sd.done) {
                long long vox;
                float len, t0;
                sd.next(vox, len, t0);
                if (len <= 0.0f)
                    continue;
                ++visits;
                int mm;
                const float rho = voxelAt<PACKED>(J, static_cast<uint32_t>(vox), mm);
                if (mm == DXMCG_TRANSPARENT_MATERIAL)
                    continue;
                const float mu = rho * lerp1(J.tot + mm * kTableNE, ec.ie, ec.fe);
                if (mu > 0.0f && acc + mu * len >= tau) {
                    hit = true;
                    v = static_cast<uint32_t>(vox);
                    m = mm;
                    thit = t0 + (tau - acc) / mu;
                    break;
                }
                acc += mu * len;
            }
        }
        if (!hit) {
            escaped = true;
            return false;
        }
        ph.px = fminf(fmaxf(fmaf(thit, ph.dx, ph.px), 0.0f), J.Lin[0]);
        ph.py = fminf(fmaxf(fmaf(thit, ph.dy, ph.py), 0.0f), J.Lin[1]);
        ph.pz = fminf(fmaxf(fmaf(thit, ph.dz, ph.pz), 0.0f), J.Lin[2]);
        return true;
    }

    // Delta tracking against the macro cell's majorant s_c mu_max(E): the sampled
    // optical depth is spent cell by cell (cell indices advance as integers, so every
    // crossing makes progress); a tentative collision in the cell is real with
    // probability mu(voxel) / (s_c mu_max).  True on a real collision.
    template <bool PACKED>
    __device__ __forceinline__ bool macroFlight(const DevJob& J, Photon& ph, Rng& rng, const EnergyCache& ec, int& cx,
        int& cy, int& cz, bool& escaped, uint32_t& v, int& m, unsigned& visits, unsigned& crossings, unsigned& err)
    {
        float tau = fmaxf(-__logf(rng.u()), 0.0f);
        const float ix = __frcp_rn(ph.dx), iy = __frcp_rn(ph.dy), iz = __frcp_rn(ph.dz);
        float muc = 0.0f;
        for (int guard = 0;; ++guard) {
            if (guard > (1 << 16)) { // cannot happen: each pass moves one cell along a fixed direction
                err |= kErrStepLimit;
                escaped = true;
                return false;
            }
            muc = __ldg(J.mscale + cx + J.mc[0] * (cy + J.mc[1] * cz)) * ec.mmax;
            float tx = FLT_MAX;
            int ax = 0;
            if (ph.dx != 0.0f) {
                const float b = fminf(static_cast<float>(cx + (ph.dx > 0.0f ? 1 : 0)) * J.cellL[0], J.L[0]);
                tx = (b - ph.px) * ix;
            }
            if (ph.dy != 0.0f) {
                const float b = fminf(static_cast<float>(cy + (ph.dy > 0.0f ? 1 : 0)) * J.cellL[1], J.L[1]);
                const float t = (b - ph.py) * iy;
                if (t < tx) {
                    tx = t;
                    ax = 1;
                }
            }
            if (ph.dz != 0.0f) {
                const float b = fminf(static_cast<float>(cz + (ph.dz > 0.0f ? 1 : 0)) * J.cellL[2], J.L[2]);
                const float t = (b - ph.pz) * iz;
                if (t < tx) {
                    tx = t;
                    ax = 2;
                }
            }
            tx = fmaxf(tx, 0.0f);
            if (tau < muc * tx) {
                const float t = tau / muc;
                ph.px = fmaf(t, ph.dx, ph.px);
                ph.py = fmaf(t, ph.dy, ph.py);
                ph.pz = fmaf(t, ph.dz, ph.pz);
                break;
            }
            tau -= muc * tx;
            ph.px = fmaf(tx, ph.dx, ph.px);
            ph.py = fmaf(tx, ph.dy, ph.py);
            ph.pz = fmaf(tx, ph.dz, ph.pz);
            ++crossings;
            bool out;
            if (ax == 0) {
                cx += ph.dx > 0.0f ? 1 : -1;
                out = cx < 0 || cx >= J.mc[0];
            } else if (ax == 1) {
                cy += ph.dy > 0.0f ? 1 : -1;
                out = cy < 0 || cy >= J.mc[1];
            } else {
                cz += ph.dz > 0.0f ? 1 : -1;
                out = cz < 0 || cz >= J.mc[2];
            }
            if (out) {
                escaped = true;
                return false;
            }
        }
        // the voxel of the tentative collision, kept inside the current cell
        const int vx = min(max(static_cast<int>(ph.px * J.isp[0]), cx * J.mb), min(cx * J.mb + J.mb, J.nx) - 1);
        const int vy = min(max(static_cast<int>(ph.py * J.isp[1]), cy * J.mb), min(cy * J.mb + J.mb, J.ny) - 1);
        const int vz = min(max(static_cast<int>(ph.pz * J.isp[2]), cz * J.mb), min(cz * J.mb + J.mb, J.nz) - 1);
        ph.px = fminf(fmaxf(ph.px, 0.0f), J.Lin[0]);
        ph.py = fminf(fmaxf(ph.py, 0.0f), J.Lin[1]);
        ph.pz = fminf(fmaxf(ph.pz, 0.0f), J.Lin[2]);
        ++visits;
        v = static_cast<uint32_t>(vx + J.nx * (vy + J.ny * vz));
        const float rho = voxelAt<PACKED>(J, v, m);
        if (m == DXMCG_TRANSPARENT_MATERIAL)
            return false;
        const float mu = rho * lerp1(J.tot + m * kTableNE, ec.ie, ec.fe);
        return rng.u() * muc < mu;
    }

    // MULTI: one queue over the concatenated history ranges of nJobs jobs (offsets[j]
    // is the first global history of job j, offsets[nJobs] the total); each lane
    // reads its job's descriptor from `jobs`.  Otherwise J0 is the only job.
    template <int TRACKING, bool PACKED, bool MULTI>
    __global__ void __launch_bounds__(256) transportKernel(const DevJob J0, const DevJob* __restrict__ jobs,
        const unsigned long long* __restrict__ offsets, int nJobs, unsigned long long h_end,
        DevCounters* __restrict__ ctr, int refillBatch, int interactBatch, int woodcockSteps)
    {
        constexpr bool BOX = TRACKING == kTrackWoodcockBox;
        constexpr bool WOODCOCK = TRACKING == DXMCG_TRACK_WOODCOCK || BOX;
        int jid = 0;
        // event counters per warp (no block-wide barrier: warps finish independently)
        __shared__ unsigned long long sCountAll[256 / 32][cNum];
        const unsigned lane = threadIdx.x & 31u;
        unsigned long long* sCount = sCountAll[threadIdx.x >> 5];
        if (lane < cNum)
            sCount[lane] = 0ull;
        __syncwarp();

        const unsigned ltMask = (1u << lane) - 1u;
        // energy sums (FP32, compensated) and the warp's history pool: in shared memory
        // for the two-region instance, whose step would spill otherwise; in registers
        // for the others, where shared memory measured slower (4 % on the 256x256x200
        // torso, 5 % on the 64-job batch, whose instance spills a little instead)
        LaneTotals<BOX> ls;
        ls.init();
        int st = kDead;
        Photon ph;
        Rng rng;
        EnergyCache ec { 0, 0.0f, 1.0f, 1.0f };
        uint32_t pv = 0; // voxel of the parked interaction
        int pm = 0;      // its material
        unsigned steps = 0, visits = 0, crossings = 0, err = 0, skipped = 0;
        int cx = 0, cy = 0, cz = 0; // macro cell of the photon (MACRO tracking)
        bool fresh = false;
        if (BOX)
            sOuterVisits[threadIdx.x] = 0u;

        for (;;) {
            const unsigned stepping = __ballot_sync(kFull, st == kStepping);
            const unsigned parked = __ballot_sync(kFull, st >= kCompton);
            const unsigned dead = ~(stepping | parked);
            const int nStep = __popc(stepping);

            // ---- refill
            if (dead && !ls.exhausted() && (__popc(dead) >= refillBatch || nStep == 0)) {
                unsigned long long poolNext, poolEnd;
                ls.loadPool(poolNext, poolEnd);
                if (poolNext >= poolEnd) {
                    unsigned long long base = 0;
                    if (lane == 0)
                        base = atomicAdd(&ctr->next, static_cast<unsigned long long>(kChunk));
                    base = __shfl_sync(kFull, base, 0);
                    if (base >= h_end) {
                        ls.markExhausted();
                        poolNext = poolEnd = 0;
                    } else {
                        poolNext = base;
                        poolEnd = min(base + kChunk, h_end);
                    }
                }
                const unsigned long long avail = poolEnd - poolNext;
                const unsigned rank = __popc(dead & ltMask);
                const bool start = st == kDead && rank < avail;
                bool entered = false;
                if (start) {
                    unsigned long long h = poolNext + rank;
                    if (MULTI) { // the queue spans all jobs: find this history's job
                        int lo = 0, hi = nJobs;
                        while (hi - lo > 1) {
                            const int mid = (lo + hi) >> 1;
                            if (__ldg(offsets + mid) <= h)
                                lo = mid;
                            else
                                hi = mid;
                        }
                        jid = lo;
                        h -= __ldg(offsets + lo);
                    }
                    const DevJob& Jr = MULTI ? jobs[jid] : J0;
                    rng.init(Jr.key, h);
                    sampleSource(Jr, h, ph, rng);
                    ls.template add<kSumSource>(ph.w * ph.E);
                    entered = enterGrid(Jr, ph);
                    if (entered) {
                        st = kStepping;
                        steps = 0;
                        fresh = true;
                        if (TRACKING == DXMCG_TRACK_SIDDON)
                            gridPos(ph.E, ec.ie, ec.fe);
                        else
                            ec.set(Jr, ph.E);
                        if (BOX && Jr.boxOn
                            && outsideBox(Jr, __float2int_rd(ph.px * Jr.isp[0]), __float2int_rd(ph.py * Jr.isp[1]),
                                __float2int_rd(ph.pz * Jr.isp[2])))
                            ec.toOuter(Jr);
                        if (TRACKING == DXMCG_TRACK_MACRO) {
                            cx = min(static_cast<int>(ph.px / Jr.cellL[0]), Jr.mc[0] - 1);
                            cy = min(static_cast<int>(ph.py / Jr.cellL[1]), Jr.mc[1] - 1);
                            cz = min(static_cast<int>(ph.pz / Jr.cellL[2]), Jr.mc[2] - 1);
                        }
                    } else {
                        ls.template add<kSumEscaped>(ph.w * ph.E);
                    }
                }
                poolNext += min(static_cast<unsigned long long>(__popc(dead)), avail);
                ls.storePool(poolNext, poolEnd);
                const unsigned mStart = __ballot_sync(kFull, start);
                const unsigned mIn = __ballot_sync(kFull, entered);
                if (lane == 0 && mStart) {
                    atomicAdd(&sCount[cHist], static_cast<unsigned long long>(__popc(mStart)));
                    atomicAdd(&sCount[cMissed], static_cast<unsigned long long>(__popc(mStart & ~mIn)));
                }
            }

            // the lane's job, after the refill may have changed it
            const DevJob& J = MULTI ? jobs[jid] : J0;

            // ---- interact
            const int nPark = __popc(parked);
            if (parked && (nPark >= interactBatch || nPark >= nStep)) {
                const bool compton = st == kCompton;
                const bool rayleigh = st == kRayleigh;
                bool cut = false, fluor = false;
                // the samplers diverge; the direction update they share runs once
                float cost = 1.0f, Ep = ph.E;
                if (compton)
                    Ep = sampleCompton(ph.E, J.mats + pm, J.ctab + pm * (kTableNE * kCTabK), ec.ie, ec.fe,
                        J.correction, rng, cost, err);
                else if (rayleigh)
                    cost = sampleRayleigh(J.rtab + pm * (kTableNE * kCTabK), ec.ie, ec.fe, rng);
                if (compton || rayleigh)
                    scatterDirection(ph.dx, ph.dy, ph.dz, cost, rng.u());
                if (compton) {
                    const float e = ph.w * (ph.E - Ep);
                    deposit(J.tally, pv, e);
                    ls.template add<kSumDeposited>(e);
                    ph.E = Ep;
                    if (Ep < 1.0f) {
                        const float r = ph.w * Ep;
                        deposit(J.tally, pv, r);
                        ls.template add<kSumDeposited>(r);
                        st = kDead;
                        cut = true;
                    } else {
                        st = kStepping;
                        if (TRACKING == DXMCG_TRACK_SIDDON)
                            gridPos(ph.E, ec.ie, ec.fe);
                        else
                            ec.set(J, ph.E);
                    }
                } else if (rayleigh) {
                    st = kStepping;
                } else if (st == kPhoto) {
                    // correction level 2: the atom may emit a K-alpha photon, which the lane
                    // follows from the absorption point in an isotropic direction
                    const float Ef = samplePhotoFluorescence(ph.E, J.mats + pm, rng);
                    const float e = ph.w * (ph.E - Ef);
                    deposit(J.tally, pv, e);
                    ls.template add<kSumDeposited>(e);
                    if (Ef > 0.0f) {
                        const float u1 = rng.u();
                        isotropicDirection(ph.dx, ph.dy, ph.dz, u1, rng.u());
                        ph.E = Ef;
                        st = kStepping;
                        fluor = true;
                        if (TRACKING == DXMCG_TRACK_SIDDON)
                            gridPos(ph.E, ec.ie, ec.fe);
                        else
                            ec.set(J, ph.E);
                    } else {
                        st = kDead;
                    }
                }
                const unsigned mC = __ballot_sync(kFull, compton);
                const unsigned mR = __ballot_sync(kFull, rayleigh);
                const unsigned mCut = __ballot_sync(kFull, cut);
                const unsigned mF = __ballot_sync(kFull, fluor);
                if (lane == 0) {
                    if (mC)
                        atomicAdd(&sCount[cCompton], static_cast<unsigned long long>(__popc(mC)));
                    if (mR)
                        atomicAdd(&sCount[cRayleigh], static_cast<unsigned long long>(__popc(mR)));
                    if (mCut)
                        atomicAdd(&sCount[cCutoff], static_cast<unsigned long long>(__popc(mCut)));
                    if (mF)
                        atomicAdd(&sCount[cFluorescence], static_cast<unsigned long long>(__popc(mF)));
                }
            }

            if (__ballot_sync(kFull, st != kDead) == 0u) {
                if (ls.exhausted())
                    break;
                continue;
            }

            // ---- step
            bool photo = false, first = false, error = false;
            if (st == kStepping) {
                bool escaped = false;
                uint32_t v = 0;
                int m = 0;
                bool real = false;
                if (WOODCOCK) {
                    // several steps per phase: most are virtual, and each phase boundary
                    // costs the warp its votes; a lane stops at a real collision or escape
                    for (int k = 0;;) {
                        real = woodcockStep<PACKED, BOX>(J, ph, rng, ec, escaped, v, m, visits, skipped);
                        if (real || escaped || ++k >= woodcockSteps)
                            break;
                        ++steps;
                    }
                } else if (TRACKING == DXMCG_TRACK_SIDDON)
                    real = siddonFlight<PACKED>(J, ph, rng, ec, escaped, v, m, visits);
                else
                    real = macroFlight<PACKED>(J, ph, rng, ec, cx, cy, cz, escaped, v, m, visits, crossings, err);
                if (escaped) {
                    ls.template add<kSumEscaped>(ph.w * ph.E);
                    st = kDead;
                } else if (real) {
                    first = fresh;
                    fresh = false;
                    const float4 a = __ldg(J.xs + m * kTableNE + ec.ie);
                    const float4 b = __ldg(J.xs + m * kTableNE + ec.ie + 1);
                    const float pe = fmaf(ec.fe, b.x - a.x, a.x);
                    const float ic = fmaf(ec.fe, b.y - a.y, a.y);
                    const float co = fmaf(ec.fe, b.z - a.z, a.z);
                    const float rt = rng.u() * (pe + ic + co);
                    if (rt < pe) {
                        photo = true;
                        if (J.correction >= 2) {
                            pv = v;
                            pm = m;
                            st = kPhoto;
                        } else {
                            const float e = ph.w * ph.E;
                            deposit(J.tally, v, e);
                            ls.template add<kSumDeposited>(e);
                            st = kDead;
                        }
                    } else {
                        pv = v;
                        pm = m;
                        st = rt < pe + ic ? kCompton : kRayleigh;
                    }
                }
                if (st != kDead && ++steps > J.maxSteps) {
                    err |= kErrStepLimit;
                    st = kDead;
                    error = true;
                }
            }
            const unsigned mPhoto = __ballot_sync(kFull, photo);
            const unsigned mFirst = __ballot_sync(kFull, first);
            const unsigned mErr = __ballot_sync(kFull, error);
            if (lane == 0) {
                if (mPhoto)
                    atomicAdd(&sCount[cPhoto], static_cast<unsigned long long>(__popc(mPhoto)));
                if (mFirst)
                    atomicAdd(&sCount[cInteracted], static_cast<unsigned long long>(__popc(mFirst)));
                if (mErr)
                    atomicAdd(&sCount[cErrors], static_cast<unsigned long long>(__popc(mErr)));
            }
        }

        // ---- flush: per-lane sums by warp, block counters by one thread
        const unsigned long long vi = warpSum(static_cast<unsigned long long>(visits));
        const unsigned long long cr = warpSum(static_cast<unsigned long long>(crossings));
        const unsigned long long sk = warpSum(static_cast<unsigned long long>(skipped));
        const unsigned long long ov = BOX ? warpSum(static_cast<unsigned long long>(sOuterVisits[threadIdx.x])) : 0ull;
        const double es = warpSum(ls.template value<kSumSource>());
        const double ee = warpSum(ls.template value<kSumEscaped>());
        const double ed = warpSum(ls.template value<kSumDeposited>());
        unsigned errAll = err;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            errAll |= __shfl_xor_sync(kFull, errAll, o);
        __syncwarp();
        if (lane == 0) {
            atomicAdd(&ctr->visits, vi);
            if (cr)
                atomicAdd(&ctr->crossings, cr);
            if (sk)
                atomicAdd(&ctr->skipped, sk);
            if (ov)
                atomicAdd(&ctr->outer, ov);
            atomicAdd(&ctr->e_source, es);
            atomicAdd(&ctr->e_escaped, ee);
            atomicAdd(&ctr->e_deposited, ed);
            if (errAll)
                atomicOr(&ctr->error_flags, errAll);
            atomicAdd(&ctr->histories, sCount[cHist]);
            atomicAdd(&ctr->missed, sCount[cMissed]);
            atomicAdd(&ctr->photo, sCount[cPhoto]);
            atomicAdd(&ctr->compton, sCount[cCompton]);
            atomicAdd(&ctr->rayleigh, sCount[cRayleigh]);
            atomicAdd(&ctr->cutoff, sCount[cCutoff]);
            atomicAdd(&ctr->errors, sCount[cErrors]);
            atomicAdd(&ctr->interacted, sCount[cInteracted]);
            if (sCount[cFluorescence])
                atomicAdd(&ctr->fluorescence, sCount[cFluorescence]);
        }
    }

} // namespace

namespace {
    using TransportFn = void (*)(const DevJob, const DevJob*, const unsigned long long*, int, unsigned long long,
        DevCounters*, int, int, int);

    // kernel instance for a tracking mode on the packed (world) or unpacked
    // (caller-owned arrays) voxel layout, single job or a batch of jobs;
    // nullptr where no instance exists
    TransportFn kernelFor(int tracking, bool packed, bool multi = false)
    {
        if (multi) {
            switch (tracking) {
            case DXMCG_TRACK_WOODCOCK: return transportKernel<DXMCG_TRACK_WOODCOCK, true, true>;
            case kTrackWoodcockBox: return transportKernel<kTrackWoodcockBox, true, true>;
            case DXMCG_TRACK_SIDDON: return transportKernel<DXMCG_TRACK_SIDDON, true, true>;
            case DXMCG_TRACK_MACRO: return transportKernel<DXMCG_TRACK_MACRO, true, true>;
            default: return nullptr;
            }
        }
        if (packed) {
            switch (tracking) {
            case DXMCG_TRACK_WOODCOCK: return transportKernel<DXMCG_TRACK_WOODCOCK, true, false>;
            case kTrackWoodcockBox: return transportKernel<kTrackWoodcockBox, true, false>;
            case DXMCG_TRACK_SIDDON: return transportKernel<DXMCG_TRACK_SIDDON, true, false>;
            case DXMCG_TRACK_MACRO: return transportKernel<DXMCG_TRACK_MACRO, true, false>;
            default: return nullptr;
            }
        }
        switch (tracking) {
        case DXMCG_TRACK_WOODCOCK: return transportKernel<DXMCG_TRACK_WOODCOCK, false, false>;
        case kTrackWoodcockBox: return transportKernel<kTrackWoodcockBox, false, false>;
        case DXMCG_TRACK_SIDDON: return transportKernel<DXMCG_TRACK_SIDDON, false, false>;
        default: return nullptr;
        }
    }

    cudaError_t launchWith(TransportFn fn, const DevJob& job, const DevJob* jobs, const unsigned long long* offsets,
        int nJobs, unsigned long long h_end, DevCounters* ctr, LaunchShape shape, cudaStream_t s)
    {
        if (!fn)
            return cudaErrorInvalidValue;
        const int refill = shape.refill_batch > 0 ? shape.refill_batch : 8;
        const int interact = shape.interact_batch > 0 ? shape.interact_batch : 8;
        const int wsteps = shape.woodcock_steps > 0 ? shape.woodcock_steps : 8;
        fn<<<shape.grid, shape.block, 0, s>>>(job, jobs, offsets, nJobs, h_end, ctr, refill, interact, wsteps);
        return cudaGetLastError();
    }

    int residentBlocks(TransportFn fn, int block)
    {
        int n = 0;
        if (!fn || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, 0) != cudaSuccess)
            return 1;
        return n > 0 ? n : 1;
    }
} // namespace

cudaError_t launchTransport(const DevJob& job, unsigned long long h_end, DevCounters* ctr, LaunchShape shape,
    cudaStream_t s)
{
    return launchWith(kernelFor(kernelTracking(job), true), job, nullptr, nullptr, 1, h_end, ctr, shape, s);
}

cudaError_t launchTransportUnpacked(const DevJob& job, unsigned long long h_end, DevCounters* ctr,
    LaunchShape shape, cudaStream_t s)
{
    return launchWith(kernelFor(kernelTracking(job), false), job, nullptr, nullptr, 1, h_end, ctr, shape, s);
}

cudaError_t launchTransportBatch(int tracking, const DevJob* jobs, const unsigned long long* offsets, int nJobs,
    unsigned long long h_end, DevCounters* ctr, LaunchShape shape, cudaStream_t s)
{
    if (!jobs || !offsets || nJobs < 1)
        return cudaErrorInvalidValue;
    const DevJob unused {};
    return launchWith(kernelFor(tracking, true, true), unused, jobs, offsets, nJobs, h_end, ctr, shape, s);
}

int transportMaxBlocksPerSMBatch(int block, int tracking) { return residentBlocks(kernelFor(tracking, true, true), block); }

int transportMaxBlocksPerSMUnpacked(int block, int tracking) { return residentBlocks(kernelFor(tracking, false), block); }

int transportMaxBlocksPerSM(int block, int tracking) { return residentBlocks(kernelFor(tracking, true), block); }

int transportRegistersPerThread(int tracking)
{
    cudaFuncAttributes a {};
    const TransportFn fn = kernelFor(tracking, true);
    return fn && cudaFuncGetAttributes(&a, fn) == cudaSuccess ? a.numRegs : -1;
}

} // namespace dxmcg
