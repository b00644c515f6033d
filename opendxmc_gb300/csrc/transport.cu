// transport.cu -- sm_103a kernels of the photon-transport hot path.
//
// One persistent kernel runs whole photon histories: every lane holds one live
// photon and advances it by one tracking step per loop iteration; lanes whose
// photon died are refilled from a warp-private pool of history indices that the
// warp takes from a global work-queue head in chunks (one atomic per chunk).
// Each history h draws its uniforms from its own Philox4x32-10 stream
// (key = seed, counter = (draw block, stream, h)), so a history's random numbers
// do not depend on which lane, warp or launch runs it.
//
// Tracking: Woodcock (delta) tracking against the majorant mu_max(E) of the
// whole grid, or regular (Siddon/Amanatides-Woo) voxel stepping with exact path
// lengths.  Interactions: photoelectric absorption, Compton (Kahn's rejection
// method for Klein-Nishina, then rejection on S(x)/Z at correction >= 1),
// Rayleigh (element choice + analytic inversion of F^2, rejection on
// (1 + cos^2)/2).  Scoring: FP64 reductions into a 32-byte per-voxel record.
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "engine.hpp"

namespace dxmcg {
namespace {

    constexpr unsigned kFull = 0xffffffffu;
    constexpr int kChunk = 256; // histories a warp takes from the queue at once
    constexpr float kMeKeV = 510.99895f;
    constexpr float kInvHc = 1.0f / 12.398419843f;

    // ---------------------------------------------------------------- Philox
    __device__ __forceinline__ void philox10(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3, uint32_t k0,
        uint32_t k1)
    {
#pragma unroll
        for (int r = 0; r < 10; ++r) {
            const uint32_t hi0 = __umulhi(0xD2511F53u, c0);
            const uint32_t lo0 = 0xD2511F53u * c0;
            const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
            const uint32_t lo1 = 0xCD9E8D57u * c2;
            const uint32_t n0 = hi1 ^ c1 ^ k0;
            const uint32_t n2 = hi0 ^ c3 ^ k1;
            c0 = n0;
            c1 = lo1;
            c2 = n2;
            c3 = lo0;
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
    }

    // (2k + 1) / 2^24 from the top 23 bits: exact in FP32 and FP64, never 0 or 1.
    __device__ __forceinline__ float toUniform(uint32_t x)
    {
        return __uint2float_rn(((x >> 9) << 1) | 1u) * 5.9604644775390625e-8f;
    }

    struct Rng {
        uint32_t k0, k1, blk, stream, lo, hi;
        uint32_t b0, b1, b2, b3;
        int left;

        __device__ void init(uint32_t key0, uint32_t key1, uint32_t s, unsigned long long h)
        {
            k0 = key0;
            k1 = key1;
            stream = s;
            lo = static_cast<uint32_t>(h);
            hi = static_cast<uint32_t>(h >> 32);
            blk = 0;
            left = 0;
        }
        __device__ __forceinline__ uint32_t raw()
        {
            if (left == 0) {
                b0 = blk;
                b1 = stream;
                b2 = lo;
                b3 = hi;
                philox10(b0, b1, b2, b3, k0, k1);
                ++blk;
                left = 4;
            }
            const uint32_t r = b0;
            b0 = b1;
            b1 = b2;
            b2 = b3;
            --left;
            return r;
        }
        __device__ __forceinline__ float u() { return toUniform(raw()); }
    };

    // Injected uniforms (sampler tests).
    struct InjectedUniforms {
        const float* p;
        int n, used;
        __device__ float u()
        {
            if (used >= n)
                return 0.5f;
            return p[used++];
        }
    };

    // ---------------------------------------------------------------- tables
    __device__ __forceinline__ void gridPos(float E, int& i, float& f)
    {
        const float x = (E - 1.0f) * 2.0f;
        int k = static_cast<int>(x);
        k = k < 0 ? 0 : (k > kTableNE - 2 ? kTableNE - 2 : k);
        i = k;
        f = x - static_cast<float>(k);
    }

    __device__ __forceinline__ float lerp1(const float* t, int i, float f)
    {
        const float a = __ldg(t + i);
        const float b = __ldg(t + i + 1);
        return fmaf(f, b - a, a);
    }

    // ---------------------------------------------------------------- samplers
    template <class U>
    __device__ float sampleCompton(float E, const DevMaterial* __restrict__ M, int correction, U& r, float& cost,
        unsigned& err)
    {
        const float k = E / kMeKeV;
        const float kk = 2.0f * k;
        for (int guard = 0; guard < kMaxRejections; ++guard) {
            const float r1 = r.u(), r2 = r.u(), r3 = r.u();
            float xm1;
            bool acc;
            if (r1 * (9.0f + kk) <= 1.0f + kk) {
                xm1 = kk * r2;
                const float x = 1.0f + xm1;
                acc = r3 * x * x <= 4.0f * xm1;
            } else {
                xm1 = kk * (1.0f - r2) / (1.0f + kk * r2);
                const float x = 1.0f + xm1;
                const float mu = 1.0f - xm1 / k;
                acc = 2.0f * r3 <= mu * mu + 1.0f / x;
            }
            if (!acc)
                continue;
            const float omu = xm1 / k;
            if (correction >= 1) {
                const float q = E * kInvHc;
                const float t = q * q * 0.5f * omu;
                const int n = M->n;
                float S = 0.0f;
                for (int i = 0; i < n; ++i) {
                    const float b = 1.0f + t / __ldg(&M->a[i]);
                    const float b2 = b * b;
                    S += __ldg(&M->nZ[i]) * (1.0f - 1.0f / (b2 * b2));
                }
                const float r4 = r.u();
                if (r4 * __ldg(&M->Zsum) > S)
                    continue;
            }
            cost = 1.0f - omu;
            return E / (1.0f + xm1);
        }
        err |= kErrRejectLimit;
        cost = 1.0f;
        return E;
    }

    template <class U>
    __device__ float sampleRayleigh(float E, const DevMaterial* __restrict__ M, U& r, unsigned& err)
    {
        const float q = E * kInvHc;
        const float T = q * q;
        const int n = M->n;
        float Gs = 0.0f;
        for (int i = 0; i < n; ++i) {
            const float a = __ldg(&M->a[i]);
            Gs += __ldg(&M->nZ2[i]) * a * (-expm1f(-3.0f * log1pf(T / a)));
        }
        for (int guard = 0; guard < kMaxRejections; ++guard) {
            const float r1 = r.u(), r2 = r.u(), r3 = r.u();
            const float target = r1 * Gs;
            float acc = 0.0f, a = 0.0f, c = 0.0f;
            for (int i = 0; i < n; ++i) {
                a = __ldg(&M->a[i]);
                c = -expm1f(-3.0f * log1pf(T / a));
                acc += __ldg(&M->nZ2[i]) * a * c;
                if (target <= acc)
                    break;
            }
            // t = a ((1 - y)^(-1/3) - 1), y = r2 c.  For y >= 1/2, 1 - y is formed as
            // (1 - r2) + r2 (1 + T/a)^-3 (1 - r2 is exact) so FP32 keeps its precision.
            const float y = r2 * c;
            float t;
            if (y < 0.5f) {
                t = a * expm1f(-log1pf(-y) / 3.0f);
            } else {
                const float omy = (1.0f - r2) + r2 * expf(-3.0f * log1pf(T / a));
                t = a * expm1f(-logf(omy) / 3.0f);
            }
            const float mu = 1.0f - 2.0f * t / T;
            if (2.0f * r3 <= 1.0f + mu * mu)
                return mu;
        }
        err |= kErrRejectLimit;
        return 1.0f;
    }

    __device__ __forceinline__ void scatterDirection(float& dx, float& dy, float& dz, float cost, float phiU)
    {
        const float sint = sqrtf(fmaxf(0.0f, 1.0f - cost * cost));
        float sp, cp;
        sincospif(2.0f * phiU, &sp, &cp);
        float nx, ny, nz;
        if (fabsf(dz) > 0.99999f) {
            nx = sint * cp;
            ny = sint * sp;
            nz = (dz > 0.0f ? 1.0f : -1.0f) * cost;
        } else {
            const float tmp = sqrtf(1.0f - dz * dz);
            const float it = 1.0f / tmp;
            nx = sint * (dx * dz * cp - dy * sp) * it + dx * cost;
            ny = sint * (dy * dz * cp + dx * sp) * it + dy * cost;
            nz = -sint * cp * tmp + dz * cost;
        }
        const float inv = rsqrtf(nx * nx + ny * ny + nz * nz);
        dx = nx * inv;
        dy = ny * inv;
        dz = nz * inv;
    }

    // ---------------------------------------------------------------- Siddon
    // Exact voxel stepping in grid-local coordinates; the FP32 operation order is
    // fixed with _rn intrinsics (no FMA contraction) so that a host restatement
    // compiled without contraction produces the same voxel sequence bit for bit.
    // Ray parameter of the crossing with the plane k * sp; the plane position is a
    // double-float (hi + fma remainder) so grazing rays do not amplify its rounding.
    __device__ __forceinline__ float crossF32(int k, float sp, float o, float d)
    {
        const float kf = __int2float_rn(k);
        const float hi = __fmul_rn(kf, sp);
        const float lo = __fmaf_rn(kf, sp, -hi);
        return __fdiv_rn(__fadd_rn(__fsub_rn(hi, o), lo), d);
    }

    struct Siddon {
        int i[3], st[3];
        float o[3], d[3], sp[3];
        float t, tmax;
        int n[3];

        // returns false if the ray misses the grid
        __device__ bool begin(const float* org, const float* dir, const int* dims, const float* spacing)
        {
            float tmin = 0.0f;
            tmax = FLT_MAX;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                n[a] = dims[a];
                sp[a] = spacing[a];
                o[a] = org[a];
                d[a] = dir[a];
                if (dir[a] != 0.0f) {
                    float t1 = crossF32(0, spacing[a], org[a], dir[a]);
                    float t2 = crossF32(dims[a], spacing[a], org[a], dir[a]);
                    if (t1 > t2) {
                        const float tt = t1;
                        t1 = t2;
                        t2 = tt;
                    }
                    if (t1 > tmin)
                        tmin = t1;
                    if (t2 < tmax)
                        tmax = t2;
                } else if (org[a] < 0.0f || org[a] >= __fmul_rn(__int2float_rn(dims[a]), spacing[a])) {
                    return false;
                }
            }
            if (!(tmin < tmax))
                return false;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float p = __fadd_rn(org[a], __fmul_rn(tmin, dir[a]));
                int k = static_cast<int>(floorf(__fdiv_rn(p, sp[a])));
                k = k < 0 ? 0 : (k > n[a] - 1 ? n[a] - 1 : k);
                i[a] = k;
                st[a] = dir[a] > 0.0f ? 1 : (dir[a] < 0.0f ? -1 : 0);
            }
            t = tmin;
            return true;
        }

        // next segment: returns false when the ray has left the grid.
        // *len may be 0 for degenerate steps (callers skip them).
        __device__ bool next(long long& voxel, float& len, float& t0)
        {
            float tn[3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
                tn[a] = st[a] != 0 ? crossF32(i[a] + (st[a] > 0 ? 1 : 0), sp[a], o[a], d[a]) : FLT_MAX;
            int ax = 0;
            if (tn[1] < tn[ax])
                ax = 1;
            if (tn[2] < tn[ax])
                ax = 2;
            const float tnext = tn[ax] < tmax ? tn[ax] : tmax;
            const float l = __fsub_rn(tnext, t);
            voxel = static_cast<long long>(i[0]) + static_cast<long long>(n[0])
                    * (static_cast<long long>(i[1]) + static_cast<long long>(n[1]) * i[2]);
            t0 = t;
            if (l > 0.0f) {
                len = l;
                t = tnext;
            } else {
                len = 0.0f;
            }
            if (tnext >= tmax) {
                done = true;
                return true;
            }
            i[ax] += st[ax];
            if (i[ax] < 0 || i[ax] >= n[ax])
                done = true;
            return true;
        }
        bool done = false;
    };

    // ---------------------------------------------------------------- photon
    struct Photon {
        float px, py, pz;
        float dx, dy, dz;
        float E, w;
    };

    struct Stats {
        unsigned histories = 0, missed = 0, visits = 0, photo = 0, compton = 0, rayleigh = 0, cutoff = 0,
                 errors = 0, interacted = 0;
        double esrc = 0.0, eesc = 0.0, edep = 0.0;
    };

    __device__ __forceinline__ void deposit(Tally* __restrict__ tally, uint32_t v, double e, Stats& st)
    {
        atomicAdd(&tally[v].e, e);
        atomicAdd(&tally[v].e2, e * e);
        atomicAdd(&tally[v].n, 1ull);
        st.edep += e;
    }

    __device__ __forceinline__ float bowtieAt(const DevBowtie* __restrict__ b, float a)
    {
        const int n = b->n;
        if (a <= b->ang[0])
            return b->w[0];
        if (a >= b->ang[n - 1])
            return b->w[n - 1];
        int lo = 0, hi = n - 1;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (b->ang[mid] <= a)
                lo = mid;
            else
                hi = mid;
        }
        const float t = (a - b->ang[lo]) / (b->ang[hi] - b->ang[lo]);
        return b->w[lo] + t * (b->w[hi] - b->w[lo]);
    }

    // Source sampling (draw order: 2 raw for the energy, fan, cone).  Leaves the
    // photon at its source position (grid-local).
    __device__ __forceinline__ void sampleSource(const DevJob& J, unsigned long long h, Photon& ph, Rng& r)
    {
        const DevExposure* __restrict__ ex = J.exps + (h / J.ppe);
        const int tube = ex->tube;
        if (J.beam_type == DXMCG_BEAM_PENCIL) {
            (void)r.raw();
            (void)r.raw();
            ph.E = J.pencil_energy;
        } else {
            const DevSpectrum* __restrict__ S = J.spec + tube;
            const uint32_t x0 = r.raw() >> 9;
            const uint32_t x1 = r.raw() >> 9;
            const int n = S->n;
            int k = static_cast<int>((static_cast<unsigned long long>(x0) * static_cast<unsigned long long>(n)) >> 23);
            k = x1 < __ldg(&S->thr[k]) ? k : __ldg(&S->alias[k]);
            ph.E = __ldg(&S->E[k]);
        }
        const float ax = (2.0f * r.u() - 1.0f) * ex->half[0];
        const float ay = (2.0f * r.u() - 1.0f) * ex->half[1];
        const float sx = sinf(ax), sy = sinf(ay);
        const float sz = sqrtf(fmaxf(0.0f, 1.0f - sx * sx - sy * sy));
        ph.dx = ex->c0[0] * sx + ex->c1[0] * sy + ex->n[0] * sz;
        ph.dy = ex->c0[1] * sx + ex->c1[1] * sy + ex->n[1] * sz;
        ph.dz = ex->c0[2] * sx + ex->c1[2] * sy + ex->n[2] * sz;
        ph.px = ex->pos[0];
        ph.py = ex->pos[1];
        ph.pz = ex->pos[2];
        float w = ex->weight;
        if (J.bowtie)
            w *= bowtieAt(J.bowtie, fabsf(ax)) * J.bowtie->inv_norm[tube];
        ph.w = w;
    }

    // Move a source photon to its entry point on the grid box; false if it misses.
    __device__ __forceinline__ bool enterGrid(const DevJob& J, Photon& ph)
    {
        float p[3] = { ph.px, ph.py, ph.pz };
        const float d[3] = { ph.dx, ph.dy, ph.dz };
        float tmin = 0.0f, tmax = FLT_MAX;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (d[a] != 0.0f) {
                const float inv = 1.0f / d[a];
                float t1 = (0.0f - p[a]) * inv, t2 = (J.L[a] - p[a]) * inv;
                if (t1 > t2) {
                    const float tt = t1;
                    t1 = t2;
                    t2 = tt;
                }
                tmin = fmaxf(tmin, t1);
                tmax = fminf(tmax, t2);
            } else if (p[a] < 0.0f || p[a] >= J.L[a]) {
                tmax = -1.0f;
            }
        }
        if (!(tmin < tmax))
            return false;
#pragma unroll
        for (int a = 0; a < 3; ++a)
            p[a] = fminf(fmaxf(p[a] + tmin * d[a], 0.0f), J.Lin[a]);
        ph.px = p[0];
        ph.py = p[1];
        ph.pz = p[2];
        return true;
    }

    // Real interaction in voxel v of material m.  Returns false if the photon died.
    __device__ __forceinline__ bool interact(const DevJob& J, uint32_t v, int m, Photon& ph, Rng& r, Stats& st,
        unsigned& err)
    {
        int ie;
        float fe;
        gridPos(ph.E, ie, fe);
        const float4 a = __ldg(J.xs + m * kTableNE + ie);
        const float4 b = __ldg(J.xs + m * kTableNE + ie + 1);
        const float ph_ = fmaf(fe, b.x - a.x, a.x);
        const float ic = fmaf(fe, b.y - a.y, a.y);
        const float co = fmaf(fe, b.z - a.z, a.z);
        const float rt = r.u() * (ph_ + ic + co);
        if (rt < ph_) {
            ++st.photo;
            deposit(J.tally, v, static_cast<double>(ph.w) * ph.E, st);
            return false;
        }
        const DevMaterial* M = J.mats + m;
        if (rt < ph_ + ic) {
            ++st.compton;
            float cost;
            const float Ep = sampleCompton(ph.E, M, J.correction, r, cost, err);
            scatterDirection(ph.dx, ph.dy, ph.dz, cost, r.u());
            deposit(J.tally, v, static_cast<double>(ph.w) * (ph.E - Ep), st);
            ph.E = Ep;
            if (ph.E < 1.0f) {
                ++st.cutoff;
                deposit(J.tally, v, static_cast<double>(ph.w) * ph.E, st);
                return false;
            }
            return true;
        }
        ++st.rayleigh;
        const float cost = sampleRayleigh(ph.E, M, r, err);
        scatterDirection(ph.dx, ph.dy, ph.dz, cost, r.u());
        return true;
    }

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

    // ---------------------------------------------------------------- transport
    __global__ void __launch_bounds__(256) transportKernel(const DevJob J, unsigned long long h_end,
        DevCounters* __restrict__ ctr)
    {
        const unsigned lane = threadIdx.x & 31u;
        const unsigned lanemaskLt = (1u << lane) - 1u;
        unsigned long long poolNext = 0, poolEnd = 0;
        bool exhausted = false;
        bool alive = false;
        Photon ph;
        Rng rng;
        Stats st;
        unsigned err = 0;
        unsigned steps = 0;
        bool fresh = false; // no real interaction yet in this history
        int ie = 0;
        float fe = 0.0f, mmax = 1.0f, invMmax = 1.0f;
        const int nx = J.nx, ny = J.ny;

        for (;;) {
            const unsigned need = __ballot_sync(kFull, !alive);
            if (need) {
                if (poolNext >= poolEnd && !exhausted) {
                    unsigned long long base = 0;
                    if (lane == 0)
                        base = atomicAdd(&ctr->next, static_cast<unsigned long long>(kChunk));
                    base = __shfl_sync(kFull, base, 0);
                    if (base >= h_end) {
                        exhausted = true;
                        poolNext = poolEnd = 0;
                    } else {
                        poolNext = base;
                        poolEnd = min(base + kChunk, h_end);
                    }
                }
                const unsigned long long avail = poolEnd - poolNext;
                const unsigned rank = __popc(need & lanemaskLt);
                if (!alive && rank < avail) {
                    const unsigned long long h = poolNext + rank;
                    rng.init(J.key0, J.key1, J.stream, h);
                    sampleSource(J, h, ph, rng);
                    ++st.histories;
                    st.esrc += static_cast<double>(ph.w) * ph.E;
                    alive = enterGrid(J, ph);
                    if (!alive) {
                        ++st.missed;
                        st.eesc += static_cast<double>(ph.w) * ph.E;
                    } else {
                        steps = 0;
                        fresh = true;
                        gridPos(ph.E, ie, fe);
                        mmax = lerp1(J.maj, ie, fe);
                        invMmax = 1.0f / mmax;
                    }
                }
                poolNext += min(static_cast<unsigned long long>(__popc(need)), avail);
            }
            if (__ballot_sync(kFull, alive) == 0u) {
                if (exhausted)
                    break;
                continue;
            }
            if (!alive)
                continue;

            if (J.tracking == DXMCG_TRACK_WOODCOCK) {
                // ---- one delta-tracking step
                const float s = -logf(rng.u()) * invMmax;
                ph.px = fmaf(s, ph.dx, ph.px);
                ph.py = fmaf(s, ph.dy, ph.py);
                ph.pz = fmaf(s, ph.dz, ph.pz);
                if (!(ph.px >= 0.0f && ph.px < J.L[0] && ph.py >= 0.0f && ph.py < J.L[1] && ph.pz >= 0.0f
                        && ph.pz < J.L[2])) {
                    st.eesc += static_cast<double>(ph.w) * ph.E;
                    alive = false;
                    continue;
                }
                ++st.visits;
                const int ix = min(static_cast<int>(ph.px * J.isp[0]), nx - 1);
                const int iy = min(static_cast<int>(ph.py * J.isp[1]), ny - 1);
                const int iz = min(static_cast<int>(ph.pz * J.isp[2]), J.nz - 1);
                const uint32_t v = static_cast<uint32_t>(ix + nx * (iy + ny * iz));
                const uint32_t word = __ldg(J.vox + v);
                const int m = static_cast<int>(word & 0xffu);
                if (m != DXMCG_TRANSPARENT_MATERIAL) {
                    const float rho = __uint_as_float(word & 0xffffff00u);
                    const float mu = rho * lerp1(J.tot + m * kTableNE, ie, fe);
                    if (rng.u() * mmax < mu) {
                        st.interacted += fresh ? 1u : 0u;
                        fresh = false;
                        const float E0 = ph.E;
                        alive = interact(J, v, m, ph, rng, st, err);
                        if (alive && ph.E != E0) {
                            gridPos(ph.E, ie, fe);
                            mmax = lerp1(J.maj, ie, fe);
                            invMmax = 1.0f / mmax;
                        }
                    }
                }
            } else {
                // ---- regular tracking: one free flight with exact voxel path lengths
                const float tau = -logf(rng.u());
                const float o[3] = { ph.px, ph.py, ph.pz };
                const float d[3] = { ph.dx, ph.dy, ph.dz };
                const int dims[3] = { J.nx, J.ny, J.nz };
                Siddon sd;
                bool hit = false;
                uint32_t hv = 0;
                int hm = 0;
                float thit = 0.0f;
                if (sd.begin(o, d, dims, J.sp)) {
                    float acc = 0.0f;
                    while (!sd.done) {
                        long long vox;
                        float len, t0;
                        sd.next(vox, len, t0);
                        if (len <= 0.0f)
                            continue;
                        ++st.visits;
                        const uint32_t word = __ldg(J.vox + vox);
                        const int m = static_cast<int>(word & 0xffu);
                        if (m == DXMCG_TRANSPARENT_MATERIAL)
                            continue;
                        const float mu = __uint_as_float(word & 0xffffff00u) * lerp1(J.tot + m * kTableNE, ie, fe);
                        if (mu > 0.0f && acc + mu * len >= tau) {
                            hit = true;
                            hv = static_cast<uint32_t>(vox);
                            hm = m;
                            thit = t0 + (tau - acc) / mu;
                            break;
                        }
                        acc += mu * len;
                    }
                }
                if (!hit) {
                    st.eesc += static_cast<double>(ph.w) * ph.E;
                    alive = false;
                    continue;
                }
                ph.px = fminf(fmaxf(fmaf(thit, ph.dx, ph.px), 0.0f), J.Lin[0]);
                ph.py = fminf(fmaxf(fmaf(thit, ph.dy, ph.py), 0.0f), J.Lin[1]);
                ph.pz = fminf(fmaxf(fmaf(thit, ph.dz, ph.pz), 0.0f), J.Lin[2]);
                st.interacted += fresh ? 1u : 0u;
                fresh = false;
                const float E0 = ph.E;
                alive = interact(J, hv, hm, ph, rng, st, err);
                if (alive && ph.E != E0)
                    gridPos(ph.E, ie, fe);
            }
            if (alive && ++steps > kMaxStepsPerHistory) {
                ++st.errors;
                err |= kErrStepLimit;
                alive = false;
            }
        }

        // ---- flush per-thread statistics (one atomic per warp and counter)
        const unsigned long long h = warpSum(static_cast<unsigned long long>(st.histories));
        const unsigned long long mi = warpSum(static_cast<unsigned long long>(st.missed));
        const unsigned long long vi = warpSum(static_cast<unsigned long long>(st.visits));
        const unsigned long long pe = warpSum(static_cast<unsigned long long>(st.photo));
        const unsigned long long co = warpSum(static_cast<unsigned long long>(st.compton));
        const unsigned long long ra = warpSum(static_cast<unsigned long long>(st.rayleigh));
        const unsigned long long cu = warpSum(static_cast<unsigned long long>(st.cutoff));
        const unsigned long long er = warpSum(static_cast<unsigned long long>(st.errors));
        const unsigned long long it = warpSum(static_cast<unsigned long long>(st.interacted));
        const double es = warpSum(st.esrc);
        const double ee = warpSum(st.eesc);
        const double ed = warpSum(st.edep);
        unsigned errAll = err;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            errAll |= __shfl_xor_sync(kFull, errAll, o);
        if (lane == 0) {
            atomicAdd(&ctr->histories, h);
            atomicAdd(&ctr->missed, mi);
            atomicAdd(&ctr->visits, vi);
            atomicAdd(&ctr->photo, pe);
            atomicAdd(&ctr->compton, co);
            atomicAdd(&ctr->rayleigh, ra);
            atomicAdd(&ctr->cutoff, cu);
            atomicAdd(&ctr->errors, er);
            atomicAdd(&ctr->interacted, it);
            atomicAdd(&ctr->e_source, es);
            atomicAdd(&ctr->e_escaped, ee);
            atomicAdd(&ctr->e_deposited, ed);
            if (errAll)
                atomicOr(&ctr->error_flags, errAll);
        }
    }

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

    __global__ void philoxKernel(int n, const uint32_t* __restrict__ c, uint32_t k0, uint32_t k1,
        uint32_t* __restrict__ out)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        uint32_t a = c[4 * i], b = c[4 * i + 1], e = c[4 * i + 2], f = c[4 * i + 3];
        philox10(a, b, e, f, k0, k1);
        out[4 * i] = a;
        out[4 * i + 1] = b;
        out[4 * i + 2] = e;
        out[4 * i + 3] = f;
    }

    __global__ void comptonKernel(int n, const float* __restrict__ E, const DevMaterial* __restrict__ M,
        int correction, const float* __restrict__ u, int stride, float* __restrict__ eo, float* __restrict__ co,
        int* __restrict__ used)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        InjectedUniforms r { u + static_cast<size_t>(i) * stride, stride, 0 };
        unsigned err = 0;
        float cost;
        eo[i] = sampleCompton(E[i], M, correction, r, cost, err);
        co[i] = cost;
        used[i] = r.used;
    }

    __global__ void rayleighKernel(int n, const float* __restrict__ E, const DevMaterial* __restrict__ M,
        const float* __restrict__ u, int stride, float* __restrict__ co, int* __restrict__ used)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        InjectedUniforms r { u + static_cast<size_t>(i) * stride, stride, 0 };
        unsigned err = 0;
        co[i] = sampleRayleigh(E[i], M, r, err);
        used[i] = r.used;
    }

    __global__ void sourceKernel(const DevJob J, unsigned long long h0, int n, float* __restrict__ out)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        Rng r;
        r.init(J.key0, J.key1, J.stream, h0 + i);
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

cudaError_t launchTransport(const DevJob& job, unsigned long long h_end, DevCounters* ctr, LaunchShape shape,
    cudaStream_t s)
{
    transportKernel<<<shape.grid, shape.block, 0, s>>>(job, h_end, ctr);
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

cudaError_t launchPhilox(int n, const uint32_t* ctr, uint32_t k0, uint32_t k1, uint32_t* out, cudaStream_t s)
{
    philoxKernel<<<(n + 255) / 256, 256, 0, s>>>(n, ctr, k0, k1, out);
    return cudaGetLastError();
}

cudaError_t launchSampleCompton(int n, const float* E, const DevMaterial* m, int correction, const float* u,
    int stride, float* e_out, float* cos_out, int* used, cudaStream_t s)
{
    comptonKernel<<<(n + 127) / 128, 128, 0, s>>>(n, E, m, correction, u, stride, e_out, cos_out, used);
    return cudaGetLastError();
}

cudaError_t launchSampleRayleigh(int n, const float* E, const DevMaterial* m, const float* u, int stride,
    float* cos_out, int* used, cudaStream_t s)
{
    rayleighKernel<<<(n + 127) / 128, 128, 0, s>>>(n, E, m, u, stride, cos_out, used);
    return cudaGetLastError();
}

cudaError_t launchSampleSource(const DevJob& job, unsigned long long h0, int n, float* out8, cudaStream_t s)
{
    sourceKernel<<<(n + 127) / 128, 128, 0, s>>>(job, h0, n, out8);
    return cudaGetLastError();
}

int transportMaxBlocksPerSM(int block)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, transportKernel, block, 0) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

int transportRegistersPerThread()
{
    cudaFuncAttributes a {};
    if (cudaFuncGetAttributes(&a, transportKernel) != cudaSuccess)
        return -1;
    return a.numRegs;
}

} // namespace dxmcg
