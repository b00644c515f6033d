// device.cuh -- device functions of the photon-transport hot path shared by the
// transport kernel and the test kernels: per-history random streams, table
// interpolation, interaction samplers, direction update, exact voxel traversal,
// source sampling.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>

#include "engine.hpp"

namespace dxmcg {
namespace dev {

    constexpr unsigned kFull = 0xffffffffu;
    constexpr float kMeKeV = 510.99895f;
    constexpr float kInvHc = 1.0f / 12.398419843f;

    // (2k + 1) / 2^24 from the top 23 bits k: exact in FP32 and FP64, never 0 or 1.
    // Formed as the float 1 + k / 2^23 (k in the mantissa) minus 1 - 2^-24; both are
    // in [1/2, 2] of each other, so the difference is exact (Sterbenz) and no
    // integer-to-float conversion is needed.
    __device__ __forceinline__ float toUniform(uint32_t x)
    {
        return __fsub_rn(__uint_as_float(0x3f800000u | (x >> 9)), 0.99999994039535522461f);
    }

    // Stream of one history: a xoshiro128+ generator (Blackman & Vigna 2018) whose
    // 128-bit state is two SplitMix64 outputs, at the counters key + (2h + 1) gamma and
    // key + (2h + 2) gamma of the run's key (the seeding the generator's authors give),
    // so every history's draws depend only on (seed, stream word, h).  Then seven 32-bit
    // ALU operations per draw with no data-dependent branch, so lanes stay converged
    // while drawing.  Every draw is used through its top 23 bits (uniforms, alias
    // columns), where the '+' output (s0 + s3) is as good as the scrambled '**' one;
    // only its lowest bits are weak, and they are never used.
    struct Rng {
        uint32_t s0, s1, s2, s3;

        __device__ __forceinline__ void init(unsigned long long key, unsigned long long h)
        {
            const unsigned long long x = key + (2ull * h + 1ull) * kGolden64;
            const unsigned long long a = splitMix64(x), b = splitMix64(x + kGolden64);
            s0 = static_cast<uint32_t>(a);
            s1 = static_cast<uint32_t>(a >> 32);
            s2 = static_cast<uint32_t>(b);
            s3 = static_cast<uint32_t>(b >> 32);
            if ((s0 | s1 | s2 | s3) == 0u)
                s0 = 0x9E3779B9u;
        }
        __device__ __forceinline__ uint32_t raw()
        {
            const uint32_t out = s0 + s3;
            const uint32_t t = s1 << 9;
            s2 ^= s0;
            s3 ^= s1;
            s1 ^= s2;
            s0 ^= s3;
            s2 ^= t;
            s3 = __funnelshift_l(s3, s3, 11);
            return out;
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
    constexpr float kCutoffKeV = 1.0f; // photons below this energy are absorbed on the spot
    constexpr int kPzTries = 32;       // electron-momentum draws per accepted scattering angle

    // Correction level 2 (impulse approximation): the scattered energy for a bound
    // electron.  A = E / E_C (E_C: the Compton line) and omu = 1 - cos(theta) come
    // from the angle already sampled.  A shell is picked by its electrons among the
    // shells bound by less than E; its projected momentum p_z = p_s t / sqrt(5) with t
    // Student-t of 5 degrees of freedom, which is the profile (1 + (p_z/p_s)^2)^-3,
    // drawn by Bailey's polar method (Math. Comp. 62, 779, 1994).  rho = p_z / m_e c
    // gives E' from the impulse-approximation energy relation (Ribberfors 1975)
    //   rho = (E E' (1 - cos) / m_e c^2 - (E - E')) / |E - E'| (photon momenta in keV),
    // solved as E'/E = (A - rho^2 cos + rho sqrt((A - cos)^2 + omu (2 - omu) (1 - rho^2)))
    //                  / (A^2 - rho^2).
    // Accepted when E' > 0 and E - E' exceeds the shell's binding; false after
    // kPzTries draws (the caller then samples a new angle).
    template <class U>
    __device__ bool dopplerEnergy(float E, float A, float omu, const DevMaterial* __restrict__ M, U& r, float& Ep)
    {
        const int ns = M->nShell;
        float tot = 0.0f;
        for (int k = 0; k < ns; ++k)
            if (__ldg(&M->shellBinding[k]) < E)
                tot += __ldg(&M->shellElectrons[k]);
        const float target = r.u() * tot;
        int sh = -1;
        float acc = 0.0f;
        for (int k = 0; k < ns; ++k) {
            if (__ldg(&M->shellBinding[k]) < E) {
                sh = k;
                acc += __ldg(&M->shellElectrons[k]);
                if (target <= acc)
                    break;
            }
        }
        if (sh < 0)
            return false;
        const float bind = __ldg(&M->shellBinding[sh]);
        const float ps = __ldg(&M->shellMomentum[sh]);
        const float c = 1.0f - omu;
        const float am = A - c;
        const float sin2 = omu * (2.0f - omu);
        for (int t = 0; t < kPzTries; ++t) {
            const float a = 2.0f * r.u() - 1.0f;
            const float b = 2.0f * r.u() - 1.0f;
            const float w = a * a + b * b;
            if (w >= 1.0f)
                continue;
            const float rho = ps * a * sqrtf((powf(w, -0.4f) - 1.0f) / w);
            const float rho2 = rho * rho;
            const float den = A * A - rho2;
            const float disc = am * am + sin2 * (1.0f - rho2);
            if (!(den > 0.0f) || !(disc >= 0.0f))
                continue;
            const float e1 = E * ((A - rho2 * c + rho * sqrtf(disc)) / den);
            if (e1 > 0.0f && E - e1 > bind) {
                Ep = e1;
                return true;
            }
        }
        return false;
    }

    // 1 - cos theta from a material's angle quantile table (row ie of tab, interpolated
    // towards row ie + 1 by fe, at the same probability): one uniform, no rejection.
    // The table's probability grid u_j = (1 - cos(pi j/(K-1)))/2 is inverted by
    // j = (K - 1) acos(1 - 2u) / pi.
    __device__ __forceinline__ float oneMinusCos(const float* __restrict__ tab, int ie, float fe, float u)
    {
        const float jf = static_cast<float>(kCTabK - 1) * 0.31830988618379067f * acosf(fmaf(-2.0f, u, 1.0f));
        const int j = min(static_cast<int>(jf), kCTabK - 2);
        const float g = jf - static_cast<float>(j);
        const float* a = tab + ie * kCTabK + j;
        const float a0 = __ldg(a), a1 = __ldg(a + 1);
        const float b0 = __ldg(a + kCTabK), b1 = __ldg(a + kCTabK + 1);
        const float lo = fmaf(g, a1 - a0, a0);
        const float hi = fmaf(g, b1 - b0, b0);
        return fmaf(fe, hi - lo, lo);
    }

    // Compton scattering: the angle from the Klein-Nishina x S table, E' from the
    // Compton relation (correction 0 and 1), or Doppler-broadened by a bound electron's
    // momentum (correction 2, which may send the draw back for a new angle).
    template <class U>
    __device__ float sampleCompton(float E, const DevMaterial* __restrict__ M, const float* __restrict__ ctab,
        int ie, float fe, int correction, U& r, float& cost, unsigned& err)
    {
        const float k = E * (1.0f / kMeKeV);
        for (int guard = 0; guard < kMaxRejections; ++guard) {
            const float omu = oneMinusCos(ctab, ie, fe, r.u());
            const float xm1 = k * omu;
            cost = 1.0f - omu;
            if (correction >= 2) {
                float Ep;
                if (!dopplerEnergy(E, 1.0f + xm1, omu, M, r, Ep))
                    continue;
                return Ep;
            }
            return E * __frcp_rn(1.0f + xm1);
        }
        err |= kErrRejectLimit;
        cost = 1.0f;
        return E;
    }

    // Rayleigh scattering: cos theta from the material's quantile table of
    // (1 + cos^2)/2 F^2(x), as for the Compton angle: one uniform, no rejection.
    template <class U>
    __device__ __forceinline__ float sampleRayleigh(const float* __restrict__ rtab, int ie, float fe, U& r)
    {
        return 1.0f - oneMinusCos(rtab, ie, fe, r.u());
    }

    // Correction level 2, photoelectric absorption: the absorbing element by its share
    // n_i Z_i^4 (/ J_K below its K edge, / J_L below its L edge) of the cross-section,
    // a K vacancy with probability 1 - 1/J_K above the element's K edge, then a K-alpha
    // photon with the element's K fluorescence yield.  Returns the fluorescence
    // energy, or 0 when no photon above the cutoff leaves the atom (all of E is then
    // deposited).  Draws: element; above the K edge the shell; for a K vacancy the
    // yield.
    __device__ __forceinline__ float photoShare(float E, const DevMaterial* __restrict__ M, int i)
    {
        float w = __ldg(&M->nZ4[i]);
        if (E < __ldg(&M->eK[i]))
            w *= __ldg(&M->invJumpK);
        if (E < __ldg(&M->eL[i]))
            w *= __ldg(&M->invJumpL);
        return w;
    }

    template <class U>
    __device__ float samplePhotoFluorescence(float E, const DevMaterial* __restrict__ M, U& r)
    {
        const int n = M->n;
        float tot = 0.0f;
        for (int i = 0; i < n; ++i)
            tot += photoShare(E, M, i);
        const float target = r.u() * tot;
        int e = n - 1;
        float acc = 0.0f;
        for (int i = 0; i < n; ++i) {
            acc += photoShare(E, M, i);
            if (target <= acc) {
                e = i;
                break;
            }
        }
        if (E < __ldg(&M->eK[e]))
            return 0.0f;
        if (r.u() >= 1.0f - __ldg(&M->invJumpK))
            return 0.0f; // L or outer shell: its fluorescence stays below the cutoff here
        if (r.u() >= __ldg(&M->omegaK[e]))
            return 0.0f; // Auger electrons: local
        const float ka = __ldg(&M->kAlpha[e]);
        return ka >= kCutoffKeV ? ka : 0.0f;
    }

    // isotropic direction from two uniforms: cos(theta) = 2 u1 - 1, phi = 2 pi u2
    __device__ __forceinline__ void isotropicDirection(float& dx, float& dy, float& dz, float u1, float u2)
    {
        const float ct = 2.0f * u1 - 1.0f;
        const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        float sp, cp;
        sincospif(2.0f * u2, &sp, &cp);
        dx = st * cp;
        dy = st * sp;
        dz = ct;
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

    // FP64 reductions into the voxel's 32-byte record (one L2 sector).
    // The deposit is formed in FP32 and widened only for the reductions.
    __device__ __forceinline__ void deposit(Tally* __restrict__ tally, uint32_t v, float e)
    {
        atomicAdd(&tally[v].e, static_cast<double>(e));
        atomicAdd(&tally[v].e2, static_cast<double>(e * e));
        atomicAdd(&tally[v].n, 1ull);
    }

    // relative bowtie weight of tube `tube` at |fan angle| a (1 when that tube has none)
    __device__ __forceinline__ float bowtieAt(const DevBowtie* __restrict__ b, int tube, float a)
    {
        const int n = b->n[tube];
        const float* __restrict__ ang = b->ang[tube];
        const float* __restrict__ w = b->w[tube];
        if (n <= 0)
            return 1.0f;
        if (a <= ang[0])
            return w[0];
        if (a >= ang[n - 1])
            return w[n - 1];
        // the segment with ang[lo] <= a < ang[lo + 1], from the cell's entry (the two
        // scans correct a cell misplaced by the rounding of a * cellScale)
        const int c = min(static_cast<int>(a * b->cellScale[tube]), kBowtieCells - 1);
        int lo = b->seg[tube][c];
        while (lo > 0 && ang[lo] > a)
            --lo;
        while (ang[lo + 1] <= a)
            ++lo;
        const int hi = lo + 1;
        const float t = (a - ang[lo]) / (ang[hi] - ang[lo]);
        return w[lo] + t * (w[hi] - w[lo]);
    }

    // exposure of history h (histories are numbered exposure-major)
    __device__ __forceinline__ unsigned exposureOf(const DevJob& J, unsigned long long h)
    {
        if ((h >> 32) == 0ull && (J.ppe >> 32) == 0ull)
            return static_cast<uint32_t>(h) / static_cast<uint32_t>(J.ppe);
        return static_cast<unsigned>(h / J.ppe);
    }

    // Source sampling (draw order: 2 raw for the energy, fan, cone).  Leaves the
    // photon at its source position (grid-local).
    __device__ __forceinline__ void sampleSource(const DevJob& J, unsigned long long h, Photon& ph, Rng& r)
    {
        // the 64-byte exposure record as four 16-byte loads: (pos, c0.x), (c0.y, c0.z,
        // c1.x, c1.y), (c1.z, n), (half, weight, tube)
        const float4* __restrict__ ex4 = reinterpret_cast<const float4*>(J.exps + exposureOf(J, h));
        const float4 q3 = __ldg(ex4 + 3);
        const int tube = __float_as_int(q3.w);
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
        const float ax = (2.0f * r.u() - 1.0f) * q3.x;
        const float ay = (2.0f * r.u() - 1.0f) * q3.y;
        // |angle| < pi/2: the hardware sine is within 2^-21.4
        const float sx = __sinf(ax), sy = __sinf(ay);
        const float sz = sqrtf(fmaxf(0.0f, 1.0f - sx * sx - sy * sy));
        const float4 q0 = __ldg(ex4), q1 = __ldg(ex4 + 1), q2 = __ldg(ex4 + 2);
        ph.dx = q0.w * sx + q1.z * sy + q2.y * sz;
        ph.dy = q1.x * sx + q1.w * sy + q2.z * sz;
        ph.dz = q1.y * sx + q2.x * sy + q2.w * sz;
        ph.px = q0.x;
        ph.py = q0.y;
        ph.pz = q0.z;
        float w = q3.z;
        if (J.bowtie)
            w *= bowtieAt(J.bowtie, tube, fabsf(ax)) * J.bowtie->inv_norm[tube];
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
                const float inv = __frcp_rn(d[a]); // the correctly rounded 1 / d, as a division gives
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

} // namespace dev
} // namespace dxmcg
