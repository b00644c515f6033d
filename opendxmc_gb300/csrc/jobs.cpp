// jobs.cpp -- see jobs.hpp.
#include "jobs.hpp"

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <utility>

namespace dxmcg {
namespace {
    constexpr double kAvogadro = 6.02214076e23;
    constexpr double kMajorantSafety = 1.0 + 1.0 / 1048576.0;

    // Element cross-section tables on the energy grid, shared by all worlds.
    struct ElementTables {
        std::vector<double> photo, incoh, coh;
    };
    std::mutex g_elementMutex;
    std::map<std::pair<int, int>, ElementTables> g_elements;

    uint64_t g_elementGeneration = ~0ull; // the physics table g_elements came from

    const ElementTables& elementTables(int Z, int correction)
    {
        std::lock_guard<std::mutex> lock(g_elementMutex);
        if (g_elementGeneration != physicsGeneration()) {
            g_elements.clear();
            g_elementGeneration = physicsGeneration();
        }
        const auto key = std::make_pair(Z, correction);
        auto it = g_elements.find(key);
        if (it != g_elements.end())
            return it->second;
        ElementTables t;
        t.photo.resize(kNE);
        t.incoh.resize(kNE);
        t.coh.resize(kNE);
        for (int i = 0; i < kNE; ++i) {
            const double E = kEmin + i * kDE;
            t.photo[i] = phys::photoelectric(E, Z);
            t.incoh[i] = phys::incoherent(E, Z, correction);
            t.coh[i] = phys::coherent(E, Z);
        }
        return g_elements.emplace(key, std::move(t)).first->second;
    }

    struct BowtieProfile {
        std::vector<double> ang, w;
        double at(double a) const
        {
            const int n = static_cast<int>(ang.size());
            if (a <= ang[0])
                return w[0];
            if (a >= ang[n - 1])
                return w[n - 1];
            int lo = 0, hi = n - 1;
            while (hi - lo > 1) {
                const int mid = (lo + hi) / 2;
                (ang[mid] <= a ? lo : hi) = mid;
            }
            const double t = (a - ang[lo]) / (ang[hi] - ang[lo]);
            return w[lo] + t * (w[hi] - w[lo]);
        }
        // exact mean over |angle| in [0, half] of the piecewise-linear profile
        double mean(double half) const
        {
            if (half <= 0)
                return 1.0;
            std::vector<double> xs { 0.0 };
            for (double a : ang)
                if (a > 0 && a < half)
                    xs.push_back(a);
            xs.push_back(half);
            double s = 0;
            for (size_t i = 0; i + 1 < xs.size(); ++i)
                s += 0.5 * (at(xs[i]) + at(xs[i + 1])) * (xs[i + 1] - xs[i]);
            return s / half;
        }
    };
} // namespace

void materialTables(const dxmcg_material& m, int correction, double* photo, double* incoh, double* coh)
{
    double wsum = 0;
    for (int i = 0; i < m.n; ++i)
        wsum += m.w[i];
    for (int e = 0; e < kNE; ++e)
        photo[e] = incoh[e] = coh[e] = 0.0;
    for (int i = 0; i < m.n; ++i) {
        const auto& t = elementTables(m.Z[i], correction);
        const double f = (m.w[i] / wsum) * kAvogadro / phys::atomicMass(m.Z[i]) * 1e-24;
        for (int e = 0; e < kNE; ++e) {
            photo[e] += f * t.photo[e];
            incoh[e] += f * t.incoh[e];
            coh[e] += f * t.coh[e];
        }
    }
}

DevMaterial toDevMaterial(const dxmcg_material& m)
{
    const auto s = samplingElements(m);
    DevMaterial d {};
    d.n = s.n;
    d.Zsum = static_cast<float>(s.Zsum);
    for (int i = 0; i < s.n; ++i) {
        d.nZ[i] = static_cast<float>(s.nZ[i]);
        d.nZ2[i] = static_cast<float>(s.nZ2[i]);
        d.a[i] = static_cast<float>(s.a[i]);
        d.ia[i] = static_cast<float>(1.0 / s.a[i]);
        d.nZ4[i] = static_cast<float>(s.nZ4[i]);
        d.eK[i] = static_cast<float>(s.eK[i]);
        d.eL[i] = static_cast<float>(s.eL[i]);
        d.kAlpha[i] = static_cast<float>(s.kAlpha[i]);
        d.omegaK[i] = static_cast<float>(s.omegaK[i]);
    }
    d.invJumpK = static_cast<float>(1.0 / phys::kJumpRatioK);
    d.invJumpL = static_cast<float>(1.0 / phys::kJumpRatioL);
    d.nShell = s.nShell;
    for (int k = 0; k < s.nShell; ++k) {
        d.shellElectrons[k] = static_cast<float>(s.shellElectrons[k]);
        d.shellBinding[k] = static_cast<float>(s.shellBinding[k]);
        d.shellMomentum[k] = static_cast<float>(s.shellMomentum[k]);
    }
    return d;
}

void buildDeviceTables(const dxmcg_material* mats, int M, int correction, const double* rhoMax, float* tot,
    float4* xs, float* maj, DevMaterial* dm)
{
    std::vector<double> mx(kNE, 0.0), ph(kNE), ic(kNE), co(kNE);
    for (int m = 0; m < M; ++m) {
        materialTables(mats[m], correction, ph.data(), ic.data(), co.data());
        for (int i = 0; i < kNE; ++i) {
            const double t = ph[i] + ic[i] + co[i];
            tot[m * kNE + i] = static_cast<float>(t);
            xs[m * kNE + i] = make_float4(static_cast<float>(ph[i]), static_cast<float>(ic[i]),
                static_cast<float>(co[i]), static_cast<float>(t));
            mx[i] = std::max(mx[i], rhoMax[m] * t);
        }
        dm[m] = toDevMaterial(mats[m]);
    }
    for (int i = 0; i < kNE; ++i)
        maj[i] = static_cast<float>(std::max(mx[i] * kMajorantSafety, 1e-30));
}

namespace {
    constexpr double kPi = 3.14159265358979323846;

    // One row of angle quantiles: 1 - cos theta at the cumulative probabilities
    // u_j = (1 - cos(pi j/(K-1)))/2, dense at both ends (the narrow peak towards
    // mu = 1 and the long backward tail of the Rayleigh distribution), for a density
    // f(1 - cos theta) on mu in [-1, 1].  The density is integrated by the trapezoid rule
    // on G equal steps of s, where w = sqrt((1 - mu)/2) = s^P (dmu = -4 w P s^(P-1) ds
    // crowds the points towards mu = 1), and each quantile is found by linear
    // interpolation of the cumulative sum.
    template <int G, int P, class F>
    void quantileRow(F density, float* row)
    {
        double cum[G + 1];
        auto weight = [&](int g) {
            const double sg = static_cast<double>(g) / G;
            const double w = P == 1 ? sg : sg * sg;
            const double dw = P == 1 ? 1.0 : 2.0 * sg;
            return density(2.0 * w * w) * 4.0 * w * dw;
        };
        cum[0] = 0.0;
        double prev = weight(0);
        for (int g = 1; g <= G; ++g) {
            const double cur = weight(g);
            cum[g] = cum[g - 1] + 0.5 * (prev + cur);
            prev = cur;
        }
        int g = 0;
        for (int j = kCTabK - 1; j >= 0; --j) { // the mass c grows as j falls
            // mass from mu = 1 down to the quantile: 1 - u_j
            const double c = 0.5 * (1.0 + std::cos(kPi * j / (kCTabK - 1))) * cum[G];
            while (g < G - 1 && cum[g + 1] < c)
                ++g;
            const double d = cum[g + 1] - cum[g];
            const double sg = (g + (d > 0.0 ? std::min(1.0, std::max(0.0, (c - cum[g]) / d)) : 0.0)) / G;
            const double w = P == 1 ? sg : sg * sg;
            row[j] = static_cast<float>(2.0 * w * w);
        }
        row[0] = 2.0f;
        row[kCTabK - 1] = 0.0f;
    }

    constexpr double kMeKeV = 510.99895, kHcKeVA = 12.398419843;

    // Compton: KN(mu) S(t(mu)) / Z (S = 1 at correction 0), 1024 steps of s = w^(1/2).
    // Kolmogorov distance of the sampled distribution from the exact one: about 1.2e-5
    // for water, 5-150 keV.
    std::vector<float> comptonAngleRows(const dxmcg_material& mat, int correction)
    {
        const auto s = samplingElements(mat);
        std::vector<float> out(static_cast<size_t>(kNE) * kCTabK);
        for (int i = 0; i < kNE; ++i) {
            const double E = kEmin + i * kDE;
            const double k = E / kMeKeV;
            const double q2 = (E / kHcKeVA) * (E / kHcKeVA);
            quantileRow<1024, 2>(
                [&](double omu) {
                    const double mu = 1.0 - omu;
                    const double P = 1.0 / (1.0 + k * omu);
                    double f = P * P * (P + 1.0 / P - 1.0 + mu * mu);
                    if (correction >= 1 && s.Zsum > 0) {
                        const double t = q2 * 0.5 * omu;
                        double S = 0.0;
                        for (int e = 0; e < s.n; ++e) {
                            const double b = 1.0 + t / s.a[e];
                            const double b2 = b * b;
                            S += s.nZ[e] * (1.0 - 1.0 / (b2 * b2));
                        }
                        f *= S / s.Zsum;
                    }
                    return f;
                },
                out.data() + static_cast<size_t>(i) * kCTabK);
        }
        return out;
    }

    // Rayleigh: (1 + mu^2)/2 sum_i n_i Z_i^2 (1 + t/a_i)^-4 with t = x^2, 1024 steps of
    // s = w^(1/2) (the distribution narrows towards mu = 1 as E grows).  Kolmogorov
    // distance about 4e-5 for water, 5-150 keV.
    std::vector<float> rayleighAngleRows(const dxmcg_material& mat)
    {
        const auto s = samplingElements(mat);
        std::vector<float> out(static_cast<size_t>(kNE) * kCTabK);
        for (int i = 0; i < kNE; ++i) {
            const double E = kEmin + i * kDE;
            const double q2 = (E / kHcKeVA) * (E / kHcKeVA);
            quantileRow<1024, 2>(
                [&](double omu) {
                    const double mu = 1.0 - omu;
                    const double t = q2 * 0.5 * omu;
                    double F2 = 0.0;
                    for (int e = 0; e < s.n; ++e) {
                        const double b = 1.0 + t / s.a[e];
                        const double b2 = b * b;
                        F2 += s.nZ2[e] / (b2 * b2);
                    }
                    return 0.5 * (1.0 + mu * mu) * F2;
                },
                out.data() + static_cast<size_t>(i) * kCTabK);
        }
        return out;
    }

    std::mutex g_angleMutex;
    std::map<std::vector<double>, std::vector<float>> g_angleRows;
    uint64_t g_angleGeneration = ~0ull;

    // kind 0: Compton at correction 0, 1: Compton at correction >= 1, 2: Rayleigh
    void angleTables(const dxmcg_material* mats, int M, int kind, float* out)
    {
        for (int m = 0; m < M; ++m) {
            std::vector<double> key { static_cast<double>(kind) };
            for (int e = 0; e < mats[m].n; ++e) {
                key.push_back(mats[m].Z[e]);
                key.push_back(mats[m].w[e]);
            }
            std::lock_guard<std::mutex> lock(g_angleMutex);
            if (g_angleGeneration != physicsGeneration()) {
                g_angleRows.clear();
                g_angleGeneration = physicsGeneration();
            }
            auto it = g_angleRows.find(key);
            if (it == g_angleRows.end())
                it = g_angleRows
                         .emplace(key, kind == 2 ? rayleighAngleRows(mats[m]) : comptonAngleRows(mats[m], kind))
                         .first;
            std::copy(it->second.begin(), it->second.end(), out + static_cast<size_t>(m) * kNE * kCTabK);
        }
    }
} // namespace

void buildComptonAngleTables(const dxmcg_material* mats, int M, int correction, float* out)
{
    angleTables(mats, M, correction >= 1 ? 1 : 0, out);
}

void buildRayleighAngleTables(const dxmcg_material* mats, int M, float* out)
{
    angleTables(mats, M, 2, out);
}

void buildBackgroundMajorant(const float* tot0, double rho0, float* out)
{
    for (int i = 0; i < kNE; ++i)
        out[i] = static_cast<float>(std::max(static_cast<double>(tot0[i]) * rho0 * kMajorantSafety, 1e-30));
}

bool twoRegionBox(const int box[6], const int32_t dims[3])
{
    return box[3] >= 0
        && (box[0] > 0 || box[1] > 0 || box[2] > 0 || box[3] < dims[0] - 1 || box[4] < dims[1] - 1
            || box[5] < dims[2] - 1);
}

double boxFraction(const int box[6], const int32_t dims[3])
{
    if (box[3] < 0)
        return 0.0;
    double f = 1.0;
    for (int a = 0; a < 3; ++a)
        f *= static_cast<double>(box[3 + a] - box[a] + 1) / dims[a];
    return f;
}

bool twoRegionFor(const dxmcg_run_options& o, double boxFrac)
{
    if (o.tracking != DXMCG_TRACK_WOODCOCK || o.two_region < 0)
        return false;
    return o.two_region > 0 || boxFrac < 0.5;
}

void setTwoRegion(DevJob& J, const int box[6], const double spacing[3], const float* majOut)
{
    J.boxOn = 1;
    J.majOut = majOut;
    for (int a = 0; a < 3; ++a) {
        J.b0[a] = box[a];
        J.bn[a] = static_cast<unsigned>(box[3 + a] - box[a] + 1);
        // the widened faces: a flight may find the box up to this much early, never late
        const double margin = std::max(1e-3, 1e-3 * spacing[a]);
        J.blo[a] = static_cast<float>(box[a] * spacing[a] - margin);
        J.bhi[a] = static_cast<float>((box[3 + a] + 1) * spacing[a] + margin);
    }
}

int buildHostJob(const dxmcg_beam& b, const int32_t dims[3], const double spacing[3], HostJob& out, std::string& err)
{
    std::vector<dxmcg_exposure> ex;
    if (expandExposures(b, ex) != DXMCG_OK || ex.empty()) {
        err = "beam: invalid geometry";
        return DXMCG_ERR_ARGUMENT;
    }
    if (b.particles_per_exposure == 0) {
        err = "beam: particles_per_exposure is 0";
        return DXMCG_ERR_ARGUMENT;
    }
    if (b.particles_per_exposure > (1ull << 40) || ex.size() > (1u << 24)) {
        err = "beam: too many histories";
        return DXMCG_ERR_ARGUMENT;
    }
    out.nHist = static_cast<uint64_t>(ex.size()) * b.particles_per_exposure;

    double origin[3];
    for (int a = 0; a < 3; ++a)
        origin[a] = -0.5 * dims[a] * spacing[a];
    out.exposures.resize(ex.size());
    for (size_t i = 0; i < ex.size(); ++i) {
        const auto& e = ex[i];
        DevExposure& d = out.exposures[i];
        const double n[3] = { e.c0[1] * e.c1[2] - e.c0[2] * e.c1[1], e.c0[2] * e.c1[0] - e.c0[0] * e.c1[2],
            e.c0[0] * e.c1[1] - e.c0[1] * e.c1[0] };
        for (int a = 0; a < 3; ++a) {
            d.pos[a] = static_cast<float>(e.pos[a] - origin[a]);
            d.c0[a] = static_cast<float>(e.c0[a]);
            d.c1[a] = static_cast<float>(e.c1[a]);
            d.n[a] = static_cast<float>(n[a]);
        }
        d.half[0] = static_cast<float>(e.half[0]);
        d.half[1] = static_cast<float>(e.half[1]);
        d.weight = static_cast<float>(e.weight);
        d.tube = e.tube;
    }

    out.spec[0] = DevSpectrum {};
    out.spec[1] = DevSpectrum {};
    if (b.type != DXMCG_BEAM_PENCIL) {
        for (int t = 0; t < 2; ++t) {
            const bool dual = b.type == DXMCG_BEAM_CT_SPIRAL_DUAL_ENERGY && t == 1;
            const auto s = tubeSpectrum(dual ? b.kvp_b : b.kvp, b.anode_angle_deg, dual ? b.n_filters_b : b.n_filters,
                dual ? b.filter_Z_b : b.filter_Z, dual ? b.filter_mm_b : b.filter_mm);
            if (s.energy.empty()) {
                if (t == 0) {
                    err = "beam: tube voltage out of range";
                    return DXMCG_ERR_ARGUMENT;
                }
                out.spec[1] = out.spec[0];
                continue;
            }
            if (s.energy.back() > kEmin + (kNE - 1) * kDE) {
                err = "beam: tube voltage above the table range (150 keV)";
                return DXMCG_ERR_ARGUMENT;
            }
            const auto at = buildAlias(s);
            DevSpectrum& d = out.spec[t];
            d.n = static_cast<int>(at.energy.size());
            for (int k = 0; k < d.n; ++k) {
                d.E[k] = at.energy[k];
                d.thr[k] = at.threshold[k];
                d.alias[k] = at.alias[k];
            }
        }
    } else if (!(b.energy_kev >= kEcut && b.energy_kev <= kEmin + (kNE - 1) * kDE)) {
        err = "beam: pencil energy out of range";
        return DXMCG_ERR_ARGUMENT;
    }

    // bowtie profiles: tube A's from n_bowtie/bowtie_*, dual-energy tube B's from
    // n_bowtie_b/bowtie_b_* (the two are set independently, beamsettingsmodel.cpp:1581-1612)
    out.hasBowtie = false;
    out.bowtie = DevBowtie {};
    const bool dualBeam = b.type == DXMCG_BEAM_CT_SPIRAL_DUAL_ENERGY;
    for (int t = 0; t < 2; ++t) {
        out.bowtie.inv_norm[t] = 1.0f;
        const int n = t == 0 ? b.n_bowtie : (dualBeam ? b.n_bowtie_b : 0);
        const double* angles = t == 0 ? b.bowtie_angle : b.bowtie_b_angle;
        const double* weights = t == 0 ? b.bowtie_weight : b.bowtie_b_weight;
        if (n <= 0 || !angles || !weights)
            continue;
        if (n > kMaxBowtie) {
            err = "beam: bowtie has too many points";
            return DXMCG_ERR_ARGUMENT;
        }
        // sorted by angle: the bowtie JSON lists points unordered (bowtiefilters.json:4-32)
        std::vector<std::pair<double, double>> pts;
        for (int i = 0; i < n; ++i)
            pts.emplace_back(angles[i], weights[i]);
        std::stable_sort(pts.begin(), pts.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
        BowtieProfile prof;
        for (const auto& p : pts) {
            prof.ang.push_back(p.first);
            prof.w.push_back(p.second);
        }
        DevBowtie& db = out.bowtie;
        db.n[t] = n;
        for (int i = 0; i < n; ++i) {
            db.ang[t][i] = static_cast<float>(prof.ang[i]);
            db.w[t][i] = static_cast<float>(prof.w[i]);
        }
        // normalised to a mean weight of 1 over the tube's fan
        double half = 0;
        for (const auto& e : ex)
            if (e.tube == t) {
                half = e.half[0];
                break;
            }
        const double m = prof.mean(half);
        db.inv_norm[t] = static_cast<float>(m > 0 ? 1.0 / m : 1.0);
        // segment index: for each cell the last segment starting at or before the cell
        const double amax = db.ang[t][n - 1];
        db.cellScale[t] = amax > 0 ? static_cast<float>(kBowtieCells / amax) : 0.0f;
        for (int c = 0; c < kBowtieCells; ++c) {
            const double a0 = amax * c / kBowtieCells;
            int k = 0;
            while (k + 1 < n - 1 && db.ang[t][k + 1] <= a0)
                ++k;
            db.seg[t][c] = static_cast<uint8_t>(k);
        }
        out.hasBowtie = true;
    }
    return DXMCG_OK;
}

void fillJobFields(DevJob& J, const dxmcg_beam& b, const dxmcg_run_options& o, const int32_t dims[3],
    const double spacing[3], int correction, int n_mats, int n_exp)
{
    J.nx = dims[0];
    J.ny = dims[1];
    J.nz = dims[2];
    for (int a = 0; a < 3; ++a) {
        J.sp[a] = static_cast<float>(spacing[a]);
        J.isp[a] = static_cast<float>(1.0 / spacing[a]);
        J.L[a] = static_cast<float>(dims[a] * spacing[a]);
        J.Lin[a] = std::nextafter(J.L[a], 0.0f);
    }
    J.n_mats = n_mats;
    J.correction = correction;
    J.n_exp = n_exp;
    J.ppe = b.particles_per_exposure;
    J.beam_type = b.type;
    J.pencil_energy = static_cast<float>(b.energy_kev);
    J.key = streamKey(o.seed, o.stream);
    J.tracking = o.tracking;
    J.maxSteps = o.max_steps > 0 ? std::min(o.max_steps, kMaxStepsPerHistory) : kMaxStepsPerHistory;
}

} // namespace dxmcg
