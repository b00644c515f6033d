// physics.cpp -- host FP64 physics model, see physics.hpp.
#include "physics.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <limits>
#include <memory>
#include <mutex>
#include <sstream>
#include <vector>

namespace dxmcg {
namespace {
    constexpr double kPi = 3.14159265358979323846;
    constexpr double kRe2Barn = 0.0794077878;   // r_e^2 in barn
    constexpr double kMeKeV = 510.99895;
    constexpr double kAvogadro = 6.02214076e23;
    constexpr double kHcKeVA = 12.398419843;    // keV * Angstrom
    constexpr double kBohrA = 0.529177210903;
    constexpr double kRydKeV = 13.605693122994e-3;
    constexpr double kPhotoC = 30.0;            // barn keV^3
    constexpr double kJumpK = phys::kJumpRatioK;
    constexpr double kJumpL = phys::kJumpRatioL;
    constexpr double kFineStructure = 7.2973525693e-3; // 1 atomic unit of momentum in m_e c
    constexpr int kQuad = 1024;                 // Simpson panels over the scattering angle

    // IUPAC abridged standard atomic weights, Z = 1..92.
    constexpr std::array<double, 93> kAtomicMass = { 0.0, 1.008, 4.0026, 6.94, 9.0122, 10.81, 12.011, 14.007,
        15.999, 18.998, 20.180, 22.990, 24.305, 26.982, 28.085, 30.974, 32.06, 35.45, 39.948, 39.098, 40.078,
        44.956, 47.867, 50.942, 51.996, 54.938, 55.845, 58.933, 58.693, 63.546, 65.38, 69.723, 72.630, 74.922,
        78.971, 79.904, 83.798, 85.468, 87.62, 88.906, 91.224, 92.906, 95.95, 98.0, 101.07, 102.91, 106.42,
        107.87, 112.41, 114.82, 118.71, 121.76, 127.60, 126.90, 131.29, 132.91, 137.33, 138.91, 140.12, 140.91,
        144.24, 145.0, 150.36, 151.96, 157.25, 158.93, 162.50, 164.93, 167.26, 168.93, 173.05, 174.97, 178.49,
        180.95, 183.84, 186.21, 190.23, 192.22, 195.08, 196.97, 200.59, 204.38, 207.2, 208.98, 209.0, 210.0,
        222.0, 223.0, 226.0, 227.0, 232.04, 231.04, 238.03 };

    double simpsonWeight(int i)
    {
        if (i == 0 || i == kQuad)
            return 1.0;
        return (i & 1) ? 4.0 : 2.0;
    }

    // Klein-Nishina differential cross-section (barn/sr per electron).
    double kleinNishinaDifferential(double k, double mu)
    {
        const double eps = 1.0 / (1.0 + k * (1.0 - mu));
        return 0.5 * kRe2Barn * eps * eps * (eps + 1.0 / eps - (1.0 - mu * mu));
    }

    std::array<double, DXMCG_MAX_ELEMENTS> normalisedWeights(const dxmcg_material& m)
    {
        std::array<double, DXMCG_MAX_ELEMENTS> w {};
        double s = 0;
        for (int i = 0; i < m.n; ++i)
            s += m.w[i];
        for (int i = 0; i < m.n; ++i)
            w[i] = s > 0 ? m.w[i] / s : 0.0;
        return w;
    }

    // ---- loaded physics tables (format in physics.hpp)
    struct ElementRecord {
        bool present = false;
        double A = 0;
        std::vector<double> photo, incoh, incohFree, coh; // at Table::energy; incohFree may be empty
        double a = 0, eK = 0, eL = 0, kAlpha = 0, omegaK = 0;
        phys::Shells shells;
    };
    struct TubeRecord {
        double kvp = 0, angle = 0;
        std::vector<double> E, w;
    };
    struct Table {
        std::vector<double> energy;
        std::array<ElementRecord, 93> el {};
        std::vector<TubeRecord> tubes;
    };
    std::mutex g_tableMutex;
    std::shared_ptr<const Table> g_table;
    std::atomic<uint64_t> g_generation { 0 };

    std::shared_ptr<const Table> currentTable()
    {
        std::lock_guard<std::mutex> lock(g_tableMutex);
        return g_table;
    }

    const ElementRecord* tableElement(const Table* t, int Z)
    {
        return (t && Z >= 1 && Z <= 92 && t->el[Z].present) ? &t->el[Z] : nullptr;
    }

    // v(E) from values at the ascending energies x (a repeated energy is an edge: the
    // value above it is the second one): the listed value at a listed energy, else
    // log-log interpolation in the bracketing interval, held at the ends.
    double tableAt(const std::vector<double>& x, const std::vector<double>& v, double E)
    {
        const size_t n = x.size();
        if (E <= x.front())
            return E == x.front() && n > 1 && x[1] == x[0] ? v[1] : v.front();
        if (E >= x.back())
            return v.back();
        // first index with x[i] > E; the interval is [i - 1, i]
        const size_t i = static_cast<size_t>(std::upper_bound(x.begin(), x.end(), E) - x.begin());
        const size_t lo = i - 1;
        if (x[lo] == E)
            return v[lo];
        const double a = v[lo], b = v[i];
        if (!(a > 0) || !(b > 0))
            return a + (b - a) * (E - x[lo]) / (x[i] - x[lo]);
        const double t = std::log(E / x[lo]) / std::log(x[i] / x[lo]);
        return std::exp(std::log(a) + t * (std::log(b) - std::log(a)));
    }
} // namespace

namespace phys {
    double atomicMass(int Z)
    {
        const auto t = currentTable();
        if (const auto* e = tableElement(t.get(), Z))
            return e->A;
        return (Z >= 1 && Z <= 92) ? kAtomicMass[Z] : 0.0;
    }

    double elementDensity(int Z)
    {
        switch (Z) {
        case 4: return 1.848;
        case 13: return 2.699;
        case 29: return 8.96;
        case 42: return 10.22;
        case 45: return 12.41;
        case 47: return 10.49;
        case 50: return 7.31;
        case 64: return 7.90;
        case 68: return 9.07;
        case 73: return 16.65;
        case 74: return 19.30;
        case 79: return 19.32;
        case 82: return 11.35;
        default: return 0.0;
        }
    }

    double formFactorScale(int Z)
    {
        const auto t = currentTable();
        if (const auto* e = tableElement(t.get(), Z))
            return e->a;
        const double x = std::cbrt(static_cast<double>(Z)) / (2.0 * kPi * kBohrA);
        return x * x;
    }

    double kleinNishinaTotal(double E)
    {
        const double k = E / kMeKeV;
        const double l = std::log1p(2.0 * k);
        const double a = (1.0 + k) / (k * k) * (2.0 * (1.0 + k) / (1.0 + 2.0 * k) - l / k);
        const double b = l / (2.0 * k);
        const double c = (1.0 + 3.0 * k) / ((1.0 + 2.0 * k) * (1.0 + 2.0 * k));
        return 2.0 * kPi * kRe2Barn * (a + b - c);
    }

    double kEdge(int Z)
    {
        const auto t = currentTable();
        if (const auto* e = tableElement(t.get(), Z))
            return e->eK;
        return kRydKeV * (Z - 1.0) * (Z - 1.0);
    }
    double lEdge(int Z)
    {
        const auto t = currentTable();
        if (const auto* e = tableElement(t.get(), Z))
            return e->eL;
        return Z > 7 ? kRydKeV * (Z - 7.4) * (Z - 7.4) * 0.25 : 0.0;
    }
    double kAlphaEnergy(int Z)
    {
        const auto t = currentTable();
        if (const auto* e = tableElement(t.get(), Z))
            return e->kAlpha;
        return 0.75 * kRydKeV * (Z - 1.0) * (Z - 1.0);
    }

    double fluorescenceYieldK(int Z)
    {
        const auto t = currentTable();
        if (const auto* e = tableElement(t.get(), Z))
            return e->omegaK;
        const double z = static_cast<double>(Z);
        const double x = 0.015 + 0.0327 * z - 0.64e-6 * z * z * z;
        const double x4 = x * x * x * x;
        return x4 / (1.0 + x4);
    }

    Shells comptonShells(int Z)
    {
        const auto t = currentTable();
        if (const auto* e = tableElement(t.get(), Z))
            return e->shells;
        Shells s;
        const double z = static_cast<double>(Z);
        const double occ[3] = { std::min(z, 2.0), std::min(std::max(z - 2.0, 0.0), 8.0), std::max(z - 10.0, 0.0) };
        const double zk = std::max(z - 1.0, 1.0);
        const double zl = std::max(z - 7.4, 0.5 * z);
        const double bind[3] = { kRydKeV * zk * zk, kRydKeV * zl * zl / 4.0, kRydKeV * (z / 3.0) * (z / 3.0) / 9.0 };
        for (int k = 0; k < 3; ++k) {
            if (occ[k] <= 0.0)
                continue;
            s.electrons[s.n] = occ[k];
            s.binding[s.n] = bind[k];
            s.momentum[s.n] = std::sqrt(bind[k] / kRydKeV) * kFineStructure;
            ++s.n;
        }
        return s;
    }

    double photoelectric(double E, int Z)
    {
        const auto t = currentTable();
        if (const auto* e = tableElement(t.get(), Z))
            return tableAt(t->energy, e->photo, E);
        const double z2 = static_cast<double>(Z) * Z;
        double s = kPhotoC * z2 * z2 / (E * E * E);
        if (E < kEdge(Z))
            s /= kJumpK;
        if (E < lEdge(Z))
            s /= kJumpL;
        return s;
    }

    // Angular integrals use t = x^2 = T (1 - mu) / 2 mapped to s in [0, 1] by t = a (B^s - 1),
    // B = 1 + T / a, which resolves the forward peak of F^2 and the rise of S.
    double incoherent(double E, int Z, int correction)
    {
        const auto tb = currentTable();
        if (const auto* e = tableElement(tb.get(), Z)) {
            if (correction >= 1)
                return tableAt(tb->energy, e->incoh, E);
            if (!e->incohFree.empty())
                return tableAt(tb->energy, e->incohFree, E);
        }
        if (correction <= 0)
            return Z * kleinNishinaTotal(E);
        const double k = E / kMeKeV;
        const double T = (E / kHcKeVA) * (E / kHcKeVA);
        const double a = formFactorScale(Z);
        const double L = std::log1p(T / a);
        double acc = 0;
        for (int i = 0; i <= kQuad; ++i) {
            const double s = static_cast<double>(i) / kQuad;
            const double t = a * std::expm1(s * L);
            const double mu = 1.0 - 2.0 * t / T;
            const double S = Z * (-std::expm1(-4.0 * s * L));
            acc += simpsonWeight(i) * kleinNishinaDifferential(k, mu) * S * a * L * std::exp(s * L);
        }
        acc *= 1.0 / (3.0 * kQuad);
        return 2.0 * kPi * (2.0 / T) * acc;
    }

    double coherent(double E, int Z)
    {
        const auto tb = currentTable();
        if (const auto* e = tableElement(tb.get(), Z))
            return tableAt(tb->energy, e->coh, E);
        const double T = (E / kHcKeVA) * (E / kHcKeVA);
        const double a = formFactorScale(Z);
        const double L = std::log1p(T / a);
        double acc = 0;
        for (int i = 0; i <= kQuad; ++i) {
            const double s = static_cast<double>(i) / kQuad;
            const double t = a * std::expm1(s * L);
            const double mu = 1.0 - 2.0 * t / T;
            acc += simpsonWeight(i) * (1.0 + mu * mu) * a * L * std::exp(-3.0 * s * L);
        }
        acc *= 1.0 / (3.0 * kQuad);
        return kPi * kRe2Barn * (2.0 / T) * static_cast<double>(Z) * Z * acc;
    }

    double knEnergyTransferFraction(double E)
    {
        const double k = E / kMeKeV;
        double num = 0, den = 0;
        for (int i = 0; i <= kQuad; ++i) {
            const double mu = -1.0 + 2.0 * static_cast<double>(i) / kQuad;
            const double eps = 1.0 / (1.0 + k * (1.0 - mu));
            const double d = kleinNishinaDifferential(k, mu) * simpsonWeight(i);
            num += d * (1.0 - eps);
            den += d;
        }
        return num / den;
    }
} // namespace phys

bool validComposition(const dxmcg_material& m)
{
    if (m.n < 1 || m.n > DXMCG_MAX_ELEMENTS)
        return false;
    double s = 0;
    for (int i = 0; i < m.n; ++i) {
        if (m.Z[i] < 1 || m.Z[i] > 92 || !(m.w[i] >= 0.0) || !std::isfinite(m.w[i]))
            return false;
        s += m.w[i];
    }
    return s > 0;
}

Attenuation attenuation(const dxmcg_material& m, int correction, double E)
{
    const auto w = normalisedWeights(m);
    Attenuation a;
    for (int i = 0; i < m.n; ++i) {
        const int Z = m.Z[i];
        const double f = w[i] * kAvogadro / phys::atomicMass(Z) * 1e-24;
        a.photo += f * phys::photoelectric(E, Z);
        a.incoherent += f * phys::incoherent(E, Z, correction);
        a.coherent += f * phys::coherent(E, Z);
    }
    return a;
}

SamplingElements samplingElements(const dxmcg_material& m)
{
    const auto w = normalisedWeights(m);
    SamplingElements s;
    s.n = m.n;
    for (int i = 0; i < m.n; ++i) {
        const double ni = w[i] / phys::atomicMass(m.Z[i]);
        s.nZ[i] = ni * m.Z[i];
        s.nZ2[i] = ni * m.Z[i] * m.Z[i];
        s.a[i] = phys::formFactorScale(m.Z[i]);
        s.Zsum += s.nZ[i];
        const double z2 = static_cast<double>(m.Z[i]) * m.Z[i];
        s.nZ4[i] = ni * z2 * z2;
        s.eK[i] = phys::kEdge(m.Z[i]);
        s.eL[i] = phys::lEdge(m.Z[i]);
        s.kAlpha[i] = phys::kAlphaEnergy(m.Z[i]);
        s.omegaK[i] = phys::fluorescenceYieldK(m.Z[i]);
        const auto sh = phys::comptonShells(m.Z[i]);
        for (int k = 0; k < sh.n; ++k) {
            s.shellElectrons[s.nShell] = ni * sh.electrons[k];
            s.shellBinding[s.nShell] = sh.binding[k];
            s.shellMomentum[s.nShell] = sh.momentum[k];
            ++s.nShell;
        }
    }
    return s;
}

namespace {
    constexpr double kTungstenKEdge = 69.525;
    constexpr std::array<double, 4> kTungstenLines = { 57.981, 59.318, 67.244, 69.067 };
    constexpr std::array<double, 4> kTungstenLineShare = { 0.27, 0.47, 0.18, 0.08 };
    constexpr double kCharacteristicYield = 0.1;

    double elementTotalUncached(int Z, double E)
    {
        dxmcg_material m {};
        m.n = 1;
        m.Z[0] = Z;
        m.w[0] = 1.0;
        return attenuation(m, 1, E).sum();
    }

    // Total mass attenuation of a filter element.  Spectra use integer energies (1 keV
    // bins); those values are computed once per element and kept (the angular
    // integrals behind them take milliseconds per spectrum otherwise).
    double elementTotal(int Z, double E)
    {
        constexpr int kMaxKeV = 512;
        static std::mutex guard;
        static std::vector<double> cache; // [Z][keV], NaN until computed
        const double k = std::floor(E);
        if (k != E || k < 1.0 || k >= kMaxKeV || Z < 1 || Z > 92)
            return elementTotalUncached(Z, E);
        const size_t idx = static_cast<size_t>(Z) * kMaxKeV + static_cast<size_t>(k);
        std::lock_guard<std::mutex> lock(guard);
        static uint64_t cacheGeneration = ~0ull; // the physics table the values came from
        if (cache.empty() || cacheGeneration != physicsGeneration()) {
            cache.assign(93 * static_cast<size_t>(kMaxKeV), std::numeric_limits<double>::quiet_NaN());
            cacheGeneration = physicsGeneration();
        }
        if (std::isnan(cache[idx]))
            cache[idx] = elementTotalUncached(Z, E);
        return cache[idx];
    }
} // namespace

Spectrum tubeSpectrum(double kvp, double anode_angle_deg, int n_filters, const int32_t* Z, const double* mm)
{
    Spectrum s;
    const int n = static_cast<int>(std::floor(kvp));
    if (n < 1 || n > 511)
        return s;
    const auto table = currentTable();
    const TubeRecord* rec = nullptr;
    if (table)
        for (const auto& t : table->tubes)
            if (t.kvp == kvp && t.angle == anode_angle_deg)
                rec = &t;
    if (rec) {
        // a loaded unfiltered spectrum of this exact tube setting
        s.energy = rec->E;
        s.weight = rec->w;
    } else {
        s.energy.resize(n);
        s.weight.resize(n);
    }
    double total = 0;
    for (int k = 0; k < n && !rec; ++k) {
        s.energy[k] = k + 1.0;
        s.weight[k] = (kvp - s.energy[k]) / s.energy[k]; // Kramers
        total += s.weight[k];
    }
    if (!rec && kvp > kTungstenKEdge) {
        const double lines = kCharacteristicYield * std::pow(kvp / kTungstenKEdge - 1.0, 1.63) * total;
        for (int l = 0; l < 4; ++l) {
            const int bin = static_cast<int>(std::floor(kTungstenLines[l] + 0.5)) - 1;
            if (bin >= 0 && bin < n)
                s.weight[bin] += lines * kTungstenLineShare[l];
        }
    }
    for (int f = 0; f < n_filters; ++f) {
        const double rho = phys::elementDensity(Z[f]);
        if (rho <= 0 || mm[f] <= 0)
            continue;
        for (size_t k = 0; k < s.energy.size(); ++k)
            s.weight[k] *= std::exp(-elementTotal(Z[f], s.energy[k]) * rho * mm[f] * 0.1);
    }
    double sum = 0;
    for (double w : s.weight)
        sum += w;
    for (double& w : s.weight)
        w = sum > 0 ? w / sum : 0.0;
    return s;
}

double tubeMeanEnergy(const Spectrum& s)
{
    double m = 0;
    for (size_t k = 0; k < s.energy.size(); ++k)
        m += s.energy[k] * s.weight[k];
    return m;
}

double airEnergyAbsorption(double E)
{
    dxmcg_material air {};
    air.n = 3;
    air.Z[0] = 7;
    air.Z[1] = 8;
    air.Z[2] = 18;
    air.w[0] = 0.755;
    air.w[1] = 0.232;
    air.w[2] = 0.013;
    const auto a = attenuation(air, 1, E);
    return a.photo + a.incoherent * phys::knEnergyTransferFraction(E);
}

double tubeAlHalfValueLayer(const Spectrum& s)
{
    const size_t n = s.energy.size();
    if (n == 0)
        return 0.0;
    std::vector<double> kerma(n), mu(n);
    double k0 = 0;
    for (size_t k = 0; k < n; ++k) {
        kerma[k] = s.weight[k] * s.energy[k] * airEnergyAbsorption(s.energy[k]);
        mu[k] = elementTotal(13, s.energy[k]) * phys::elementDensity(13) * 0.1;
        k0 += kerma[k];
    }
    double lo = 0, hi = 100;
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        double t = 0;
        for (size_t k = 0; k < n; ++k)
            t += kerma[k] * std::exp(-mu[k] * mid);
        (t > 0.5 * k0 ? lo : hi) = mid;
    }
    return 0.5 * (lo + hi);
}

// Vose's construction of Walker's alias table.
AliasTable buildAlias(const Spectrum& s)
{
    const int n = static_cast<int>(s.weight.size());
    AliasTable t;
    t.energy.resize(n);
    t.threshold.resize(n);
    t.alias.resize(n);
    std::vector<double> p(n), prob(n, 1.0);
    std::vector<int> small, large;
    double sum = 0;
    for (double w : s.weight)
        sum += w;
    for (int i = 0; i < n; ++i) {
        p[i] = s.weight[i] / sum * n;
        t.alias[i] = i;
        t.energy[i] = static_cast<float>(s.energy[i]);
    }
    for (int i = 0; i < n; ++i)
        (p[i] < 1.0 ? small : large).push_back(i);
    while (!small.empty() && !large.empty()) {
        const int l = small.back();
        small.pop_back();
        const int g = large.back();
        large.pop_back();
        prob[l] = p[l];
        t.alias[l] = g;
        p[g] = (p[g] + p[l]) - 1.0;
        (p[g] < 1.0 ? small : large).push_back(g);
    }
    for (int i = 0; i < n; ++i)
        t.threshold[i] = static_cast<uint32_t>(std::floor(prob[i] * 8388608.0 + 0.5));
    return t;
}


// ---------------------------------------------------------------- physics tables
namespace {
    bool readValues(std::istream& in, size_t n, std::vector<double>& out)
    {
        out.resize(n);
        for (size_t i = 0; i < n; ++i)
            if (!(in >> out[i]) || !std::isfinite(out[i]) || out[i] < 0)
                return false;
        return true;
    }

    // the file's tokens with comments removed
    bool tokens(const std::string& path, std::stringstream& out)
    {
        std::ifstream f(path);
        if (!f)
            return false;
        std::string line;
        while (std::getline(f, line)) {
            const auto c = line.find('#');
            out << (c == std::string::npos ? line : line.substr(0, c)) << '\n';
        }
        return true;
    }
} // namespace

uint64_t physicsGeneration() { return g_generation.load(); }

void resetPhysicsTable()
{
    std::lock_guard<std::mutex> lock(g_tableMutex);
    g_table.reset();
    ++g_generation;
}

int loadPhysicsTable(const std::string& path, std::string& err)
{
    std::stringstream in;
    if (!tokens(path, in)) {
        err = "cannot read " + path;
        return DXMCG_ERR_ARGUMENT;
    }
    auto t = std::make_shared<Table>();
    std::string word;
    int version = 0;
    if (!(in >> word) || word != "dxmcg-physics" || !(in >> version) || version != 1) {
        err = "not a dxmcg-physics 1 table";
        return DXMCG_ERR_ARGUMENT;
    }
    while (in >> word) {
        if (word == "energies") {
            size_t n = 0;
            if (!(in >> n) || n < 2 || n > 100000 || !readValues(in, n, t->energy)) {
                err = "bad energies line";
                return DXMCG_ERR_ARGUMENT;
            }
            for (size_t i = 0; i < n; ++i)
                if (!(t->energy[i] > 0) || (i > 0 && t->energy[i] < t->energy[i - 1])
                    || (i > 1 && t->energy[i] == t->energy[i - 2])) {
                    err = "energies must be positive and ascending (an energy at most twice)";
                    return DXMCG_ERR_ARGUMENT;
                }
        } else if (word == "element") {
            int Z = 0;
            double A = 0;
            if (!(in >> Z >> A) || Z < 1 || Z > 92 || !(A > 0)) {
                err = "bad element line";
                return DXMCG_ERR_ARGUMENT;
            }
            if (t->energy.empty()) {
                err = "element before energies";
                return DXMCG_ERR_ARGUMENT;
            }
            ElementRecord e;
            e.A = A;
            bool photo = false, incoh = false, coh = false, ff = false, edges = false, fl = false, sh = false;
            const size_t n = t->energy.size();
            while (in >> word && word != "end") {
                bool ok = true;
                if (word == "photo")
                    ok = photo = readValues(in, n, e.photo);
                else if (word == "incoherent")
                    ok = incoh = readValues(in, n, e.incoh);
                else if (word == "incoherent_free")
                    ok = readValues(in, n, e.incohFree);
                else if (word == "coherent")
                    ok = coh = readValues(in, n, e.coh);
                else if (word == "formfactor")
                    ok = ff = static_cast<bool>(in >> e.a) && e.a > 0;
                else if (word == "edges")
                    ok = edges = static_cast<bool>(in >> e.eK >> e.eL) && e.eK >= 0 && e.eL >= 0;
                else if (word == "fluorescence")
                    ok = fl = static_cast<bool>(in >> e.kAlpha >> e.omegaK) && e.kAlpha >= 0 && e.omegaK >= 0
                        && e.omegaK <= 1;
                else if (word == "shells") {
                    ok = static_cast<bool>(in >> e.shells.n) && e.shells.n >= 0 && e.shells.n <= 3;
                    for (int k = 0; ok && k < e.shells.n; ++k)
                        ok = static_cast<bool>(in >> e.shells.electrons[k] >> e.shells.binding[k]
                                 >> e.shells.momentum[k])
                            && e.shells.electrons[k] >= 0 && e.shells.binding[k] >= 0 && e.shells.momentum[k] > 0;
                    sh = ok;
                } else {
                    err = "unknown element field '" + word + "'";
                    return DXMCG_ERR_ARGUMENT;
                }
                if (!ok) {
                    err = "bad '" + word + "' of element " + std::to_string(Z);
                    return DXMCG_ERR_ARGUMENT;
                }
            }
            if (word != "end" || !(photo && incoh && coh && ff && edges && fl && sh)) {
                err = "element " + std::to_string(Z)
                    + " needs photo, incoherent, coherent, formfactor, edges, fluorescence, shells and end";
                return DXMCG_ERR_ARGUMENT;
            }
            e.present = true;
            t->el[Z] = std::move(e);
        } else if (word == "tube") {
            TubeRecord r;
            size_t m = 0;
            if (!(in >> r.kvp >> r.angle >> m) || !(r.kvp > 1) || m < 1 || m > 512) {
                err = "bad tube line";
                return DXMCG_ERR_ARGUMENT;
            }
            r.E.resize(m);
            r.w.resize(m);
            for (size_t i = 0; i < m; ++i)
                if (!(in >> r.E[i] >> r.w[i]) || !(r.E[i] >= 1.0) || r.E[i] > r.kvp || !(r.w[i] >= 0)) {
                    err = "bad tube entry";
                    return DXMCG_ERR_ARGUMENT;
                }
            t->tubes.push_back(std::move(r));
        } else {
            err = "unknown table entry '" + word + "'";
            return DXMCG_ERR_ARGUMENT;
        }
    }
    std::lock_guard<std::mutex> lock(g_tableMutex);
    g_table = std::move(t);
    ++g_generation;
    return DXMCG_OK;
}

int writePhysicsTable(const std::string& path, int n, const int32_t* Zs, std::string& err)
{
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) {
        err = "cannot write " + path;
        return DXMCG_ERR_ARGUMENT;
    }
    std::fprintf(f, "# photon interaction data for the dxmcg engine, written by dxmcg_physics_write\n");
    std::fprintf(f, "dxmcg-physics 1\nenergies %d", kNE);
    for (int i = 0; i < kNE; ++i)
        std::fprintf(f, " %.17g", kEmin + i * kDE);
    std::fprintf(f, "\n");
    const auto row = [&](const char* name, auto fn) {
        std::fprintf(f, "  %s", name);
        for (int i = 0; i < kNE; ++i)
            std::fprintf(f, " %.17g", fn(kEmin + i * kDE));
        std::fprintf(f, "\n");
    };
    for (int k = 0; k < n; ++k) {
        const int Z = Zs[k];
        if (Z < 1 || Z > 92)
            continue;
        std::fprintf(f, "element %d %.17g\n", Z, phys::atomicMass(Z));
        row("photo", [Z](double E) { return phys::photoelectric(E, Z); });
        row("incoherent", [Z](double E) { return phys::incoherent(E, Z, 1); });
        row("incoherent_free", [Z](double E) { return phys::incoherent(E, Z, 0); });
        row("coherent", [Z](double E) { return phys::coherent(E, Z); });
        std::fprintf(f, "  formfactor %.17g\n  edges %.17g %.17g\n  fluorescence %.17g %.17g\n",
            phys::formFactorScale(Z), phys::kEdge(Z), phys::lEdge(Z), phys::kAlphaEnergy(Z),
            phys::fluorescenceYieldK(Z));
        const auto sh = phys::comptonShells(Z);
        std::fprintf(f, "  shells %d", sh.n);
        for (int s = 0; s < sh.n; ++s)
            std::fprintf(f, " %.17g %.17g %.17g", sh.electrons[s], sh.binding[s], sh.momentum[s]);
        std::fprintf(f, "\nend\n");
    }
    const bool ok = std::fclose(f) == 0;
    if (!ok)
        err = "error writing " + path;
    return ok ? DXMCG_OK : DXMCG_ERR_ARGUMENT;
}

} // namespace dxmcg
