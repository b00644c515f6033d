/*
 * dxmc_oracle.c -- FP64 CPU restatement of the photon-transport hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  PARITY UNPINNED
 * against DXMClib, which the reference does not contain (CMakeLists.txt:68-75);
 * see dxmc_oracle.h for what each part restates.
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off, no fast-math: the FP32
 * Siddon restatement below must round exactly like the device traversal).
 */
#include "dxmc_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* Physical constants                                                         */
/* ------------------------------------------------------------------------- */
#define PI 3.14159265358979323846
#define R_E2_BARN 0.0794077878 /* classical electron radius squared, barn */
#define ME_KEV 510.99895
#define N_A 6.02214076e23
#define HC_KEV_A 12.398419843 /* h c in keV * Angstrom */
#define BOHR_A 0.529177210903
#define RYD_KEV 13.605693122994e-3
/* project-authored photoelectric model constants (see or_sigma_photo) */
#define C_PE 30.0
#define J_K 7.0
#define J_L 3.0
#define QUAD_N 1024
#define E_CUT 1.0
#define MAX_STEPS 1000000

/* Standard atomic weights (g/mol), Z = 1..92 (IUPAC abridged values). */
static const double ATOMIC_MASS[93] = { 0.0, 1.008, 4.0026, 6.94, 9.0122, 10.81, 12.011, 14.007,
    15.999, 18.998, 20.180, 22.990, 24.305, 26.982, 28.085, 30.974, 32.06, 35.45, 39.948, 39.098,
    40.078, 44.956, 47.867, 50.942, 51.996, 54.938, 55.845, 58.933, 58.693, 63.546, 65.38, 69.723,
    72.630, 74.922, 78.971, 79.904, 83.798, 85.468, 87.62, 88.906, 91.224, 92.906, 95.95, 98.0,
    101.07, 102.91, 106.42, 107.87, 112.41, 114.82, 118.71, 121.76, 127.60, 126.90, 131.29, 132.91,
    137.33, 138.91, 140.12, 140.91, 144.24, 145.0, 150.36, 151.96, 157.25, 158.93, 162.50, 164.93,
    167.26, 168.93, 173.05, 174.97, 178.49, 180.95, 183.84, 186.21, 190.23, 192.22, 195.08, 196.97,
    200.59, 204.38, 207.2, 208.98, 209.0, 210.0, 222.0, 223.0, 226.0, 227.0, 232.04, 231.04,
    238.03 };

/* ------------------------------------------------------------------------- */
/* Physics tables: the engine's "dxmcg-physics 1" text format (documented in the  */
/* engine's csrc/physics.hpp), restated.  A loaded table replaces the model's     */
/* numbers for the elements and tube settings it lists.  Not thread-safe against */
/* running transports: load before building worlds.                              */
/* ------------------------------------------------------------------------- */
typedef struct {
    int present;
    double A;
    double *photo, *incoh, *incoh_free, *coh; /* at TABLE.energy; incoh_free may be NULL */
    double a, eK, eL, kAlpha, omegaK;
    int nsh;
    double sh_el[3], sh_bd[3], sh_mo[3];
} elem_rec;
typedef struct {
    double kvp, angle;
    int m;
    double *E, *w;
} tube_rec;
static struct {
    int n;
    double* energy;
    elem_rec el[93];
    int ntubes;
    tube_rec* tubes;
} TABLE;

static const elem_rec* table_elem(int Z)
{
    return (Z >= 1 && Z <= 92 && TABLE.el[Z].present) ? &TABLE.el[Z] : NULL;
}

/* the listed value at a listed energy (the second of a repeated one: above the
 * edge), else log-log interpolation in the bracketing interval, held at the ends */
static double table_at(const double* v, double E)
{
    const double* x = TABLE.energy;
    const int n = TABLE.n;
    if (E <= x[0])
        return (E == x[0] && n > 1 && x[1] == x[0]) ? v[1] : v[0];
    if (E >= x[n - 1])
        return v[n - 1];
    int lo = 0, hi = n; /* first index with x > E */
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (x[mid] > E)
            hi = mid;
        else
            lo = mid + 1;
    }
    const int i = lo, l = i - 1;
    if (x[l] == E)
        return v[l];
    const double a = v[l], b = v[i];
    if (!(a > 0) || !(b > 0))
        return a + (b - a) * (E - x[l]) / (x[i] - x[l]);
    const double t = log(E / x[l]) / log(x[i] / x[l]);
    return exp(log(a) + t * (log(b) - log(a)));
}

void or_physics_reset(void)
{
    for (int Z = 0; Z <= 92; ++Z) {
        free(TABLE.el[Z].photo);
        free(TABLE.el[Z].incoh);
        free(TABLE.el[Z].incoh_free);
        free(TABLE.el[Z].coh);
    }
    for (int t = 0; t < TABLE.ntubes; ++t) {
        free(TABLE.tubes[t].E);
        free(TABLE.tubes[t].w);
    }
    free(TABLE.tubes);
    free(TABLE.energy);
    memset(&TABLE, 0, sizeof(TABLE));
}

typedef struct {
    char* p; /* next unread character */
} toks;
/* the next whitespace-separated word (terminated in place), or NULL at the end */
static char* tok(toks* t)
{
    char* c = t->p;
    while (*c == ' ' || *c == '\t' || *c == '\r' || *c == '\n')
        ++c;
    if (!*c) {
        t->p = c;
        return NULL;
    }
    char* w = c;
    while (*c && *c != ' ' && *c != '\t' && *c != '\r' && *c != '\n')
        ++c;
    if (*c)
        *c++ = '\0';
    t->p = c;
    return w;
}
static int num(toks* t, double* out)
{
    char* w = tok(t);
    char* end = NULL;
    if (!w)
        return 0;
    *out = strtod(w, &end);
    return *end == '\0' && isfinite(*out);
}
static double* values(toks* t, int n)
{
    double* v = (double*)malloc((size_t)n * sizeof(double));
    for (int i = 0; v && i < n; ++i)
        if (!num(t, &v[i]) || v[i] < 0) {
            free(v);
            return NULL;
        }
    return v;
}

/* 0 on success; a negative value (nothing changed) on a malformed file */
int or_physics_load(const char* path)
{
    FILE* f = fopen(path, "rb");
    if (!f)
        return -1;
    fseek(f, 0, SEEK_END);
    const long len = ftell(f);
    fseek(f, 0, SEEK_SET);
    char* buf = (char*)malloc((size_t)len + 1);
    const size_t got = fread(buf, 1, (size_t)len, f);
    fclose(f);
    buf[got] = '\0';
    for (char* c = buf; *c; ++c) /* comments run to the end of the line */
        if (*c == '#')
            while (*c && *c != '\n')
                *c++ = ' ';
    or_physics_reset();
    toks t = { buf };
    char* w = tok(&t);
    double v;
    int rc = 0;
    if (!w || strcmp(w, "dxmcg-physics") != 0 || !num(&t, &v) || v != 1.0)
        rc = -2;
    while (rc == 0 && (w = tok(&t)) != NULL) {
        if (strcmp(w, "energies") == 0) {
            if (!num(&t, &v) || v < 2) {
                rc = -3;
                break;
            }
            TABLE.n = (int)v;
            TABLE.energy = values(&t, TABLE.n);
            if (!TABLE.energy)
                rc = -3;
            for (int i = 0; rc == 0 && i < TABLE.n; ++i) /* ascending, an energy at most twice */
                if (!(TABLE.energy[i] > 0) || (i > 0 && TABLE.energy[i] < TABLE.energy[i - 1])
                    || (i > 1 && TABLE.energy[i] == TABLE.energy[i - 2]))
                    rc = -3;
        } else if (strcmp(w, "element") == 0) {
            double z, A;
            if (!num(&t, &z) || !num(&t, &A) || z < 1 || z > 92 || !(A > 0) || TABLE.n == 0) {
                rc = -4;
                break;
            }
            elem_rec* e = &TABLE.el[(int)z];
            e->A = A;
            int seen = 0; /* formfactor, edges, fluorescence, shells */
            while (rc == 0 && (w = tok(&t)) != NULL && strcmp(w, "end") != 0) {
                if (strcmp(w, "formfactor") == 0 || strcmp(w, "edges") == 0 || strcmp(w, "fluorescence") == 0
                    || strcmp(w, "shells") == 0)
                    seen |= w[0] == 'f' ? (w[1] == 'o' ? 1 : 4) : (w[0] == 'e' ? 2 : 8);
                if (strcmp(w, "photo") == 0)
                    rc = (e->photo = values(&t, TABLE.n)) ? 0 : -5;
                else if (strcmp(w, "incoherent") == 0)
                    rc = (e->incoh = values(&t, TABLE.n)) ? 0 : -5;
                else if (strcmp(w, "incoherent_free") == 0)
                    rc = (e->incoh_free = values(&t, TABLE.n)) ? 0 : -5;
                else if (strcmp(w, "coherent") == 0)
                    rc = (e->coh = values(&t, TABLE.n)) ? 0 : -5;
                else if (strcmp(w, "formfactor") == 0)
                    rc = num(&t, &e->a) ? 0 : -5;
                else if (strcmp(w, "edges") == 0)
                    rc = num(&t, &e->eK) && num(&t, &e->eL) ? 0 : -5;
                else if (strcmp(w, "fluorescence") == 0)
                    rc = num(&t, &e->kAlpha) && num(&t, &e->omegaK) ? 0 : -5;
                else if (strcmp(w, "shells") == 0) {
                    rc = num(&t, &v) && v >= 0 && v <= 3 ? 0 : -5;
                    e->nsh = (int)v;
                    for (int k = 0; rc == 0 && k < e->nsh; ++k)
                        rc = num(&t, &e->sh_el[k]) && num(&t, &e->sh_bd[k]) && num(&t, &e->sh_mo[k]) ? 0 : -5;
                } else
                    rc = -6;
            }
            if (rc == 0 && (!w || !e->photo || !e->incoh || !e->coh || seen != 15 || !(e->a > 0)))
                rc = -7;
            e->present = rc == 0;
        } else if (strcmp(w, "tube") == 0) {
            double kvp, ang, m;
            if (!num(&t, &kvp) || !num(&t, &ang) || !num(&t, &m) || m < 1 || m > 512) {
                rc = -8;
                break;
            }
            TABLE.tubes = (tube_rec*)realloc(TABLE.tubes, (size_t)(TABLE.ntubes + 1) * sizeof(tube_rec));
            tube_rec* r = &TABLE.tubes[TABLE.ntubes++];
            r->kvp = kvp;
            r->angle = ang;
            r->m = (int)m;
            r->E = (double*)malloc((size_t)r->m * sizeof(double));
            r->w = (double*)malloc((size_t)r->m * sizeof(double));
            for (int i = 0; rc == 0 && i < r->m; ++i)
                rc = num(&t, &r->E[i]) && num(&t, &r->w[i]) ? 0 : -8;
        } else
            rc = -9;
    }
    free(buf);
    if (rc != 0)
        or_physics_reset();
    return rc;
}

double or_atomic_mass(int Z)
{
    const elem_rec* e = table_elem(Z);
    if (e)
        return e->A;
    return (Z >= 1 && Z <= 92) ? ATOMIC_MASS[Z] : 0.0;
}

/* Mass densities (g/cm3) of elements used as tube filters. */
double or_element_density(int Z)
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

/* ------------------------------------------------------------------------- */
/* Physics model (project-authored, parametric; DXMClib's Livermore tables are
 * not available).  Per atom, in barn, E in keV.
 *  - Compton: Klein-Nishina; with correction >= 1 (simulationwidget.cpp:71-73,
 *    "Livermore") the differential cross-section is multiplied by the
 *    incoherent scattering function S(x, Z).
 *  - Rayleigh: Thomson cross-section times the atomic form factor F(x, Z)^2.
 *  - F and S use one hydrogen-like orbital scaled by the Thomas-Fermi radius:
 *    F = Z / (1 + x^2/a_Z)^2, S = Z (1 - (F/Z)^2), a_Z = (Z^(1/3) / (2 pi a0))^2,
 *    x = sin(theta/2) / lambda in 1/Angstrom.
 *  - Photoelectric: C_PE Z^4 / E^3 with K and L edges at Moseley energies
 *    (Ryd (Z-1)^2 and Ryd (Z-7.4)^2 / 4) and jump ratios J_K, J_L.           */
/* ------------------------------------------------------------------------- */
static double a_Z(int Z)
{
    const double x = cbrt((double)Z) / (2.0 * PI * BOHR_A);
    return x * x;
}

double or_sigma_kn(double E)
{
    const double k = E / ME_KEV;
    const double l = log1p(2.0 * k);
    const double a = (1.0 + k) / (k * k) * (2.0 * (1.0 + k) / (1.0 + 2.0 * k) - l / k);
    const double b = l / (2.0 * k);
    const double c = (1.0 + 3.0 * k) / ((1.0 + 2.0 * k) * (1.0 + 2.0 * k));
    return 2.0 * PI * R_E2_BARN * (a + b - c);
}

/* Klein-Nishina d sigma / d Omega per electron (barn/sr) at cos(theta) = mu. */
static double kn_dcs(double k, double mu)
{
    const double eps = 1.0 / (1.0 + k * (1.0 - mu));
    return 0.5 * R_E2_BARN * eps * eps * (eps + 1.0 / eps - (1.0 - mu * mu));
}

/* Correction level 2 element data (project model, independent restatement):
 * K edge Ryd (Z-1)^2, L edge Ryd (Z-7.4)^2/4 (Z > 7), K-alpha 0.75 Ryd (Z-1)^2, K
 * fluorescence yield omega = X^4/(1+X^4), X = 0.015 + 0.0327 Z - 0.64e-6 Z^3
 * (Bambynek et al., Rev. Mod. Phys. 44, 716, 1972).  Compton shells: K with
 * min(Z,2) electrons bound by Ryd max(Z-1,1)^2; L with up to 8 electrons bound by
 * Ryd max(Z-7.4, Z/2)^2/4; the rest bound by Ryd (Z/3)^2/9; each with the
 * hydrogen-like 1s Compton profile of momentum scale sqrt(U/Ryd) atomic units
 * (alpha m_e c per atomic unit). */
#define FINE_STRUCTURE 7.2973525693e-3
double or_k_edge(int Z)
{
    const elem_rec* e = table_elem(Z);
    return e ? e->eK : RYD_KEV * (Z - 1.0) * (Z - 1.0);
}
double or_l_edge(int Z)
{
    const elem_rec* e = table_elem(Z);
    if (e)
        return e->eL;
    return Z > 7 ? RYD_KEV * (Z - 7.4) * (Z - 7.4) * 0.25 : 0.0;
}
double or_k_alpha(int Z)
{
    const elem_rec* e = table_elem(Z);
    return e ? e->kAlpha : 0.75 * RYD_KEV * (Z - 1.0) * (Z - 1.0);
}
double or_fluorescence_yield_k(int Z)
{
    const elem_rec* e = table_elem(Z);
    if (e)
        return e->omegaK;
    const double x = 0.015 + 0.0327 * Z - 0.64e-6 * (double)Z * Z * Z;
    const double x4 = x * x * x * x;
    return x4 / (1.0 + x4);
}
int or_compton_shells(int Z, double electrons[3], double binding[3], double momentum[3])
{
    const elem_rec* e = table_elem(Z);
    if (e) {
        for (int k = 0; k < e->nsh; ++k) {
            electrons[k] = e->sh_el[k];
            binding[k] = e->sh_bd[k];
            momentum[k] = e->sh_mo[k];
        }
        return e->nsh;
    }
    const double z = (double)Z;
    double occ[3], bind[3];
    occ[0] = z < 2.0 ? z : 2.0;
    occ[1] = z - 2.0 < 0.0 ? 0.0 : (z - 2.0 > 8.0 ? 8.0 : z - 2.0);
    occ[2] = z - 10.0 < 0.0 ? 0.0 : z - 10.0;
    const double zk = z - 1.0 > 1.0 ? z - 1.0 : 1.0;
    const double zl = z - 7.4 > 0.5 * z ? z - 7.4 : 0.5 * z;
    bind[0] = RYD_KEV * zk * zk;
    bind[1] = RYD_KEV * zl * zl / 4.0;
    bind[2] = RYD_KEV * (z / 3.0) * (z / 3.0) / 9.0;
    int n = 0;
    for (int k = 0; k < 3; ++k) {
        if (occ[k] <= 0.0)
            continue;
        electrons[n] = occ[k];
        binding[n] = bind[k];
        momentum[n] = sqrt(bind[k] / RYD_KEV) * FINE_STRUCTURE;
        ++n;
    }
    return n;
}

double or_sigma_photo(double E, int Z)
{
    const elem_rec* e = table_elem(Z);
    if (e)
        return table_at(e->photo, E);
    const double z2 = (double)Z * (double)Z;
    double s = C_PE * z2 * z2 / (E * E * E);
    const double ek = RYD_KEV * (Z - 1.0) * (Z - 1.0);
    const double el = Z > 7 ? RYD_KEV * (Z - 7.4) * (Z - 7.4) * 0.25 : 0.0;
    if (E < ek)
        s /= J_K;
    if (E < el)
        s /= J_L;
    return s;
}

/* Integrals over the scattering angle use t = x^2 = t_max (1 - mu) / 2 mapped as
 * t = a (B^s - 1), B = 1 + t_max / a, s in [0, 1], composite Simpson, QUAD_N panels. */
static double simpson_weight(int i)
{
    if (i == 0 || i == QUAD_N)
        return 1.0;
    return (i & 1) ? 4.0 : 2.0;
}

double or_sigma_incoh(double E, int Z, int correction)
{
    const elem_rec* e = table_elem(Z);
    if (e && correction >= 1)
        return table_at(e->incoh, E);
    if (e && e->incoh_free)
        return table_at(e->incoh_free, E);
    if (correction <= 0)
        return Z * or_sigma_kn(E);
    const double k = E / ME_KEV;
    const double T = (E / HC_KEV_A) * (E / HC_KEV_A);
    const double a = a_Z(Z);
    const double L = log1p(T / a);
    double acc = 0.0;
    for (int i = 0; i <= QUAD_N; ++i) {
        const double s = (double)i / QUAD_N;
        const double t = a * expm1(s * L);
        const double mu = 1.0 - 2.0 * t / T;
        const double S = Z * (-expm1(-4.0 * s * L));
        acc += simpson_weight(i) * kn_dcs(k, mu) * S * a * L * exp(s * L);
    }
    acc *= 1.0 / (3.0 * QUAD_N);
    return 2.0 * PI * (2.0 / T) * acc;
}

double or_sigma_coh(double E, int Z)
{
    const elem_rec* e = table_elem(Z);
    if (e)
        return table_at(e->coh, E);
    const double T = (E / HC_KEV_A) * (E / HC_KEV_A);
    const double a = a_Z(Z);
    const double L = log1p(T / a);
    double acc = 0.0;
    for (int i = 0; i <= QUAD_N; ++i) {
        const double s = (double)i / QUAD_N;
        const double t = a * expm1(s * L);
        const double mu = 1.0 - 2.0 * t / T;
        acc += simpson_weight(i) * (1.0 + mu * mu) * a * L * exp(-3.0 * s * L);
    }
    acc *= 1.0 / (3.0 * QUAD_N);
    return PI * R_E2_BARN * (2.0 / T) * (double)Z * (double)Z * acc;
}

/* Mean fraction of the photon energy given to the free electron in a
 * Klein-Nishina collision (for the air-kerma weighting of the HVL). */
double or_kn_energy_transfer_fraction(double E)
{
    const double k = E / ME_KEV;
    double num = 0.0, den = 0.0;
    for (int i = 0; i <= QUAD_N; ++i) {
        const double mu = -1.0 + 2.0 * (double)i / QUAD_N;
        const double eps = 1.0 / (1.0 + k * (1.0 - mu));
        const double d = kn_dcs(k, mu) * simpson_weight(i);
        num += d * (1.0 - eps);
        den += d;
    }
    return num / den;
}

static void normalised(const or_composition* c, double* w)
{
    double s = 0.0;
    for (int i = 0; i < c->n; ++i)
        s += c->w[i];
    for (int i = 0; i < c->n; ++i)
        w[i] = s > 0 ? c->w[i] / s : 0.0;
}

void or_attenuation(const or_composition* c, int correction, int n, const double* E, double* photo,
    double* incoh, double* coh)
{
    double w[OR_MAX_ELEMENTS];
    normalised(c, w);
    for (int j = 0; j < n; ++j) {
        double p = 0, ic = 0, co = 0;
        for (int i = 0; i < c->n; ++i) {
            const int Z = c->Z[i];
            const double f = w[i] * N_A / or_atomic_mass(Z) * 1e-24;
            p += f * or_sigma_photo(E[j], Z);
            ic += f * or_sigma_incoh(E[j], Z, correction);
            co += f * or_sigma_coh(E[j], Z);
        }
        photo[j] = p;
        incoh[j] = ic;
        coh[j] = co;
    }
}

static double element_mu_rho(int Z, double E)
{
    or_composition c = { 1, { Z }, { 1.0 } };
    double p, i, co;
    or_attenuation(&c, 1, 1, &E, &p, &i, &co);
    return p + i + co;
}

/* ------------------------------------------------------------------------- */
/* Tube (ctsegmentationpipeline.cpp:66-71; beamsettingsmodel.cpp:257-330):
 * Kramers' thick-target law N(E) ~ (kVp - E) / E on 1 keV bins, tungsten K lines
 * (K edge 69.525 keV) with Green-Cosslett (kVp/E_K - 1)^1.63 yield scaling, and
 * exponential filtration by each added filter.  Anode angle is carried but the
 * model has no heel/self-absorption term.                                    */
/* ------------------------------------------------------------------------- */
#define W_K_EDGE 69.525
static const double W_LINES[4] = { 57.981, 59.318, 67.244, 69.067 };
static const double W_LINE_FRAC[4] = { 0.27, 0.47, 0.18, 0.08 };
#define C_CHAR 0.1

int or_tube_spectrum(double kvp, double anode_angle_deg, int n_filters, const int32_t* fZ,
    const double* fmm, double* energies, double* weights, int cap)
{
    int n = (int)floor(kvp);
    if (n < 1 || n > cap)
        return -1;
    const tube_rec* rec = NULL; /* a loaded unfiltered spectrum of this exact setting */
    for (int t = 0; t < TABLE.ntubes; ++t)
        if (TABLE.tubes[t].kvp == kvp && TABLE.tubes[t].angle == anode_angle_deg)
            rec = &TABLE.tubes[t];
    double total = 0.0;
    if (rec) {
        if (rec->m > cap)
            return -1;
        n = rec->m;
        memcpy(energies, rec->E, (size_t)n * sizeof(double));
        memcpy(weights, rec->w, (size_t)n * sizeof(double));
    } else
        for (int k = 0; k < n; ++k) {
            const double E = k + 1.0;
            energies[k] = E;
            weights[k] = (kvp - E) / E;
            total += weights[k];
        }
    if (!rec && kvp > W_K_EDGE) {
        const double nchar = C_CHAR * pow(kvp / W_K_EDGE - 1.0, 1.63) * total;
        for (int l = 0; l < 4; ++l) {
            const int bin = (int)floor(W_LINES[l] + 0.5) - 1;
            if (bin >= 0 && bin < n)
                weights[bin] += nchar * W_LINE_FRAC[l];
        }
    }
    for (int f = 0; f < n_filters; ++f) {
        const double rho = or_element_density(fZ[f]);
        if (rho <= 0.0 || fmm[f] <= 0.0)
            continue;
        for (int k = 0; k < n; ++k)
            weights[k] *= exp(-element_mu_rho(fZ[f], energies[k]) * rho * fmm[f] * 0.1);
    }
    double s = 0.0;
    for (int k = 0; k < n; ++k)
        s += weights[k];
    for (int k = 0; k < n; ++k)
        weights[k] = s > 0 ? weights[k] / s : 0.0;
    return n;
}

double or_tube_mean_energy(double kvp, int n_filters, const int32_t* fZ, const double* fmm)
{
    double E[512], w[512];
    const int n = or_tube_spectrum(kvp, 12.0, n_filters, fZ, fmm, E, w, 512);
    double m = 0.0;
    for (int k = 0; k < n; ++k)
        m += E[k] * w[k];
    return m;
}

/* Air (dry, by mass): N 75.5 %, O 23.2 %, Ar 1.3 %. */
static const or_composition AIR = { 3, { 7, 8, 18 }, { 0.755, 0.232, 0.013 } };

double or_tube_al_hvl_mm(double kvp, int n_filters, const int32_t* fZ, const double* fmm)
{
    double E[512], w[512], ph[512], ic[512], co[512], kw[512], mal[512];
    const int n = or_tube_spectrum(kvp, 12.0, n_filters, fZ, fmm, E, w, 512);
    if (n <= 0)
        return 0.0;
    or_attenuation(&AIR, 1, n, E, ph, ic, co);
    double k0 = 0.0;
    for (int k = 0; k < n; ++k) {
        kw[k] = w[k] * E[k] * (ph[k] + ic[k] * or_kn_energy_transfer_fraction(E[k]));
        mal[k] = element_mu_rho(13, E[k]) * or_element_density(13) * 0.1; /* per mm */
        k0 += kw[k];
    }
    double lo = 0.0, hi = 100.0;
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        double s = 0.0;
        for (int k = 0; k < n; ++k)
            s += kw[k] * exp(-mal[k] * mid);
        if (s > 0.5 * k0)
            lo = mid;
        else
            hi = mid;
    }
    return 0.5 * (lo + hi);
}

/* Analytic dose calibration (calibration.cpp in the engine; the trailing `true` of
 * transport(world, beam, progress, true), simulationpipeline.cpp:165): the factor
 * applied to every history weight so that the N = n_hist histories of the beam
 * deliver its target.  DX / CBCT: the dose-area product per photon of a point source
 * is E (mu_tr/rho)_air at any distance (setDAPvalue, beamsettingsmodel.cpp:576);
 * pencil: the air kerma of one photon per cm2 is E (mu_tr/rho)_air (setAirKerma,
 * beamsettingsmodel.cpp:675).  1 without a target; -1 for CT beams (their factor
 * comes from a CTDI phantom simulation, not restated here). */
double or_calibration_factor(const or_beam* b, uint64_t n_hist)
{
    const double k = 1.602176634e-10; /* mGy g / keV */
    if (n_hist == 0)
        return 1.0;
    if (b->type == OR_BEAM_DX || b->type == OR_BEAM_CBCT) {
        if (!(b->dap_mgycm2 > 0.0))
            return 1.0;
        double E[512], w[512], ph[512], ic[512], co[512];
        const int n = or_tube_spectrum(b->kvp, b->anode_angle_deg, b->n_filters, b->filter_Z, b->filter_mm, E, w, 512);
        if (n <= 0)
            return 1.0;
        or_attenuation(&AIR, 1, n, E, ph, ic, co);
        double per = 0.0;
        for (int i = 0; i < n; ++i)
            per += w[i] * E[i] * (ph[i] + ic[i] * or_kn_energy_transfer_fraction(E[i]));
        return b->dap_mgycm2 / ((double)n_hist * per * k);
    }
    if (b->type == OR_BEAM_PENCIL) {
        if (!(b->air_kerma_mgy > 0.0))
            return 1.0;
        const double E = b->energy_kev;
        double ph, ic, co;
        or_attenuation(&AIR, 1, 1, &E, &ph, &ic, &co);
        return b->air_kerma_mgy / ((double)n_hist * E * (ph + ic * or_kn_energy_transfer_fraction(E)) * k);
    }
    return -1.0;
}

/* ------------------------------------------------------------------------- */
/* Per-history streams                                                         */
/* ------------------------------------------------------------------------- */
/* The output function of SplitMix64 (Steele, Lea & Flood, OOPSLA 2014). */
static inline uint64_t splitmix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
#define GOLDEN64 0x9E3779B97F4A7C15ull

/* the key of a run's streams, a mix of (seed, stream word) */
static inline uint64_t stream_key(uint64_t seed, uint32_t stream)
{
    return splitmix64(seed ^ splitmix64((uint64_t)stream + GOLDEN64));
}

/* (2 k + 1) / 2^24 with k the top 23 bits: exactly representable in FP32, in (0, 1). */
double or_uniform_from_u32(uint32_t x) { return (double)((x >> 9) * 2u + 1u) * (1.0 / 16777216.0); }

/* Draw source: either the stream of one history, or injected uniforms.
 * History h's stream: the 128-bit state of a xoshiro128+ generator (Blackman & Vigna,
 * "Scrambled linear pseudorandom number generators", 2018; output s0 + s3, of which
 * only the top 23 bits are ever used) is two SplitMix64 outputs at the counters
 * key + (2h + 1) gamma and key + (2h + 2) gamma, key = stream_key(seed, stream) (the
 * seeding the generator's authors give), so every history's draws depend only on
 * (seed, stream, h). */
typedef struct {
    uint32_t s[4];
    const double* inj;
    int n_inj, used;
} rng_t;

static void rng_stream(rng_t* r, uint64_t seed, uint32_t stream, uint64_t hist)
{
    const uint64_t x = stream_key(seed, stream) + (2ull * hist + 1ull) * GOLDEN64;
    const uint64_t a = splitmix64(x), b = splitmix64(x + GOLDEN64);
    r->s[0] = (uint32_t)a;
    r->s[1] = (uint32_t)(a >> 32);
    r->s[2] = (uint32_t)b;
    r->s[3] = (uint32_t)(b >> 32);
    if ((r->s[0] | r->s[1] | r->s[2] | r->s[3]) == 0u)
        r->s[0] = 0x9E3779B9u; /* the all-zero state is the generator's fixed point */
    r->inj = NULL;
    r->used = 0;
}

static inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

static uint32_t rng_raw(rng_t* r)
{
    uint32_t* s = r->s;
    const uint32_t out = s[0] + s[3];
    const uint32_t t = s[1] << 9;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl32(s[3], 11);
    r->used++;
    return out;
}

static double rng_u(rng_t* r)
{
    if (r->inj) {
        if (r->used >= r->n_inj)
            return 0.5; /* exhausted: callers size the array generously */
        return r->inj[r->used++];
    }
    return or_uniform_from_u32(rng_raw(r));
}

/* ------------------------------------------------------------------------- */
/* Vector helpers                                                              */
/* ------------------------------------------------------------------------- */
static void cross3(const double a[3], const double b[3], double c[3])
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static void normalise3(double v[3])
{
    const double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (n > 0) {
        v[0] /= n;
        v[1] /= n;
        v[2] /= n;
    }
}

/* Rodrigues rotation of v about unit axis k by angle a (right-handed). */
static void rotate3(const double v[3], const double k[3], double a, double out[3])
{
    double kxv[3];
    cross3(k, v, kxv);
    const double kv = k[0] * v[0] + k[1] * v[1] + k[2] * v[2];
    const double c = cos(a), s = sin(a);
    for (int i = 0; i < 3; ++i)
        out[i] = v[i] * c + kxv[i] * s + k[i] * kv * (1.0 - c);
}

/* ------------------------------------------------------------------------- */
/* Beam -> exposures.  DX: every exposure has the beam's pose
 * (dxmc_specialization.cpp:78-90 sets position/cosines; collimation half-angles
 * :123-129).  Rotating beams place the source at SDD/2 from the isocentre, the
 * fan along c0, the rotation axis along c1, and direction = c0 x c1 pointing at
 * the isocentre (beamactorcontainer.cpp:44-67 uses the same basis).         */
/* ------------------------------------------------------------------------- */
static double interp_profile(const double* w, int n, double f)
{
    /* w sampled uniformly on [0, 1] */
    if (n <= 0)
        return 1.0;
    if (n == 1)
        return w[0];
    double x = f * (n - 1);
    if (x <= 0)
        return w[0];
    if (x >= n - 1)
        return w[n - 1];
    const int i = (int)x;
    const double t = x - i;
    return w[i] + t * (w[i + 1] - w[i]);
}

static double aec_weight(const or_beam* b, double z)
{
    if (b->n_aec <= 0 || !b->aec_weight)
        return 1.0;
    const double z0 = b->aec_start[2], z1 = b->aec_stop[2];
    const double f = (z1 != z0) ? (z - z0) / (z1 - z0) : 0.0;
    return interp_profile(b->aec_weight, b->n_aec, f);
}

static void rotating_exposure(const double iso[3], const double axis_in[3], double angle, double sid,
    double half_fan, double half_cone, or_exposure* e)
{
    double axis[3] = { axis_in[0], axis_in[1], axis_in[2] };
    normalise3(axis);
    const double xh[3] = { 1, 0, 0 }, yh[3] = { 0, 1, 0 };
    double s0[3];
    cross3(axis, xh, s0);
    if (s0[0] * s0[0] + s0[1] * s0[1] + s0[2] * s0[2] < 1e-12)
        cross3(axis, yh, s0);
    normalise3(s0);
    double s[3];
    rotate3(s0, axis, angle, s);
    double n[3] = { -s[0], -s[1], -s[2] };
    for (int i = 0; i < 3; ++i) {
        e->pos[i] = iso[i] + sid * s[i];
        e->c1[i] = axis[i];
    }
    cross3(axis, n, e->c0);
    e->half[0] = half_fan;
    e->half[1] = half_cone;
    e->weight = 1.0;
    e->tube = 0;
}

/* Organ AEC: tube output lowered to `low` over the gantry sector [start, stop]
 * (degrees, counter-clockwise, wrapping), ramped back to 1 over `ramp` degrees on
 * both sides; with compensation the exposures outside are raised to keep the mean. */
static double wrap360(double a)
{
    a = fmod(a, 360.0);
    return a < 0 ? a + 360.0 : a;
}

static void organ_aec(const or_beam* b, const double* gantry, or_exposure* out, int n)
{
    if (!b->organ_aec || n <= 0)
        return;
    double low = b->organ_aec_low_weight;
    low = low < 0.0 ? 0.0 : (low > 1.0 ? 1.0 : low);
    const double ramp = b->organ_aec_ramp_deg > 0.0 ? b->organ_aec_ramp_deg : 0.0;
    const double s0 = wrap360(b->organ_aec_start_deg);
    const double span = wrap360(b->organ_aec_stop_deg - b->organ_aec_start_deg);
    double* f = (double*)malloc(n * sizeof(double));
    double lowered = 0.0;
    int n_out = 0;
    for (int i = 0; i < n; ++i) {
        const double d = wrap360(gantry[i] - s0);
        if (d <= span) {
            f[i] = low;
        } else {
            const double a = d - span, c = 360.0 - d;
            const double dist = a < c ? a : c;
            f[i] = dist < ramp ? low + (1.0 - low) * dist / ramp : 1.0;
        }
        if (f[i] < 1.0)
            lowered += f[i];
        else
            n_out++;
    }
    if (b->organ_aec_compensate && n_out > 0) {
        const double raise = ((double)n - lowered) / (double)n_out;
        for (int i = 0; i < n; ++i)
            if (f[i] >= 1.0)
                f[i] = raise;
    }
    for (int i = 0; i < n; ++i)
        out[i].weight *= f[i];
    free(f);
}

int or_beam_exposures(const or_beam* b, or_exposure* out, int cap)
{
    double gantry[1 << 14];
    int n = 0;
    const double zaxis[3] = { 0, 0, 1 };
    if (b->type == OR_BEAM_DX || b->type == OR_BEAM_PENCIL) {
        n = (int)(b->n_exposures > 0 ? b->n_exposures : 1);
        if (!out)
            return n;
        if (n > cap)
            return -n;
        for (int i = 0; i < n; ++i) {
            or_exposure* e = &out[i];
            memcpy(e->pos, b->position, sizeof(e->pos));
            memcpy(e->c0, b->cosines[0], sizeof(e->c0));
            memcpy(e->c1, b->cosines[1], sizeof(e->c1));
            if (b->type == OR_BEAM_PENCIL) {
                e->half[0] = e->half[1] = 0.0;
            } else {
                e->half[0] = b->half_angles[0];
                e->half[1] = b->half_angles[1];
            }
            e->weight = 1.0;
            e->tube = 0;
        }
        return n;
    }
    const double sid = 0.5 * b->sdd_cm;
    const double step = b->step_angle_deg * PI / 180.0;
    const double a0 = b->start_angle_deg * PI / 180.0;
    if (b->type == OR_BEAM_CT_SPIRAL || b->type == OR_BEAM_CT_SPIRAL_DUAL) {
        const double dz = b->stop[2] - b->start[2];
        const double feed = b->collimation_cm * b->pitch; /* cm per rotation */
        const double per_rot = 2.0 * PI / step;
        long m = (long)ceil(fabs(dz) / feed * per_rot - 1e-9);
        if (m < 1)
            m = 1;
        const int dual = b->type == OR_BEAM_CT_SPIRAL_DUAL;
        n = (int)(dual ? 2 * m : m);
        if (n > (1 << 14))
            return 0; /* the oracle records at most 16384 gantry angles */
        if (!out)
            return n;
        if (n > cap)
            return -n;
        const double half_cone = atan(0.5 * b->collimation_cm / sid);
        for (long i = 0; i < m; ++i) {
            const double ang = a0 + i * step;
            const double z = b->start[2] + (dz >= 0 ? 1.0 : -1.0) * (double)i / per_rot * feed;
            const double iso[3] = { b->start[0], b->start[1], z };
            for (int t = 0; t < (dual ? 2 : 1); ++t) {
                or_exposure* e = &out[dual ? 2 * i + t : i];
                const double fov = (t == 1) ? b->fov_b_cm : b->scan_fov_cm;
                rotating_exposure(iso, zaxis, ang + (t == 1 ? 0.5 * PI : 0.0), sid, atan(0.5 * fov / sid),
                    half_cone, e);
                e->tube = t;
                const double tw = dual ? (t == 0 ? 2.0 * b->tube_a_weight : 2.0 * (1.0 - b->tube_a_weight)) : 1.0;
                e->weight = aec_weight(b, z) * tw;
                gantry[dual ? 2 * i + t : i] = (ang + (t == 1 ? 0.5 * PI : 0.0)) * 180.0 / PI;
            }
        }
    } else if (b->type == OR_BEAM_CT_SEQUENTIAL) {
        const long per_rot = lround(2.0 * PI / step);
        const int slices = b->n_slices > 0 ? b->n_slices : 1;
        n = (int)(per_rot * slices);
        if (n > (1 << 14))
            return 0; /* the oracle records at most 16384 gantry angles */
        if (!out)
            return n;
        if (n > cap)
            return -n;
        const double half_cone = atan(0.5 * b->collimation_cm / sid);
        for (int s = 0; s < slices; ++s) {
            const double iso[3] = { b->position[0], b->position[1], b->position[2] + s * b->slice_spacing_cm };
            for (long i = 0; i < per_rot; ++i) {
                or_exposure* e = &out[s * per_rot + i];
                rotating_exposure(iso, zaxis, a0 + i * step, sid, atan(0.5 * b->scan_fov_cm / sid), half_cone, e);
                e->weight = aec_weight(b, iso[2]);
                gantry[s * per_rot + i] = (a0 + i * step) * 180.0 / PI;
            }
        }
    } else if (b->type == OR_BEAM_CBCT) {
        const double a1 = b->stop_angle_deg * PI / 180.0;
        long m = (long)floor((a1 - a0) / step + 1e-9) + 1;
        if (m < 1)
            m = 1;
        n = (int)m;
        if (n > (1 << 14))
            return 0; /* the oracle records at most 16384 gantry angles */
        if (!out)
            return n;
        if (n > cap)
            return -n;
        for (long i = 0; i < m; ++i) {
            rotating_exposure(b->position, b->rotation_axis, a0 + i * step, sid, b->half_angles[0],
                b->half_angles[1], &out[i]);
            gantry[i] = (a0 + i * step) * 180.0 / PI;
        }
    } else {
        return 0;
    }
    /* AEC weights are relative: mean over exposures = 1 */
    if (b->type != OR_BEAM_CBCT) {
        double s = 0.0;
        for (int i = 0; i < n; ++i)
            s += out[i].weight;
        const double mean = s / n;
        if (mean > 0)
            for (int i = 0; i < n; ++i)
                out[i].weight /= mean;
    }
    organ_aec(b, gantry, out, n);
    return n;
}

/* ------------------------------------------------------------------------- */
/* Siddon / Amanatides-Woo traversal in grid-local coordinates (grid spans
 * [0, n_a * sp_a) on each axis).  The FP32 variant fixes the operation order so
 * that the device traversal reproduces it bit for bit.                        */
/* ------------------------------------------------------------------------- */
/* Ray parameter where the ray o + t d crosses the plane at k * sp.  The plane
 * position is carried as a double-float (hi + fma remainder) so that its FP32
 * rounding is not amplified by 1/|d| on grazing rays: the result is within about
 * one ulp of t.  Division, not a rounded reciprocal. */
static float cross_f32(int k, float sp, float o, float d)
{
    const float kf = (float)k;
    const float hi = kf * sp;
    const float lo = fmaf(kf, sp, -hi);
    return ((hi - o) + lo) / d;
}

int or_siddon_f32(const float o[3], const float d[3], const int32_t n[3], const float sp[3], int cap,
    int64_t* idx, float* len)
{
    float tmin = 0.0f, tmax = FLT_MAX;
    for (int a = 0; a < 3; ++a) {
        if (d[a] != 0.0f) {
            float t1 = cross_f32(0, sp[a], o[a], d[a]);
            float t2 = cross_f32(n[a], sp[a], o[a], d[a]);
            if (t1 > t2) {
                const float tt = t1;
                t1 = t2;
                t2 = tt;
            }
            if (t1 > tmin)
                tmin = t1;
            if (t2 < tmax)
                tmax = t2;
        } else if (o[a] < 0.0f || o[a] >= (float)n[a] * sp[a]) {
            return 0;
        }
    }
    if (!(tmin < tmax))
        return 0;
    int i[3], st[3];
    for (int a = 0; a < 3; ++a) {
        const float p = o[a] + tmin * d[a];
        int k = (int)floorf(p / sp[a]);
        if (k < 0)
            k = 0;
        if (k > n[a] - 1)
            k = n[a] - 1;
        i[a] = k;
        st[a] = d[a] > 0.0f ? 1 : (d[a] < 0.0f ? -1 : 0);
    }
    float t = tmin;
    int cnt = 0;
    for (;;) {
        float tn[3];
        for (int a = 0; a < 3; ++a)
            tn[a] = st[a] != 0 ? cross_f32(i[a] + (st[a] > 0 ? 1 : 0), sp[a], o[a], d[a]) : FLT_MAX;
        int ax = 0;
        if (tn[1] < tn[ax])
            ax = 1;
        if (tn[2] < tn[ax])
            ax = 2;
        float tnext = tn[ax] < tmax ? tn[ax] : tmax;
        const float l = tnext - t;
        if (l > 0.0f) {
            if (cnt < cap) {
                idx[cnt] = (int64_t)i[0] + (int64_t)n[0] * ((int64_t)i[1] + (int64_t)n[1] * i[2]);
                len[cnt] = l;
            }
            cnt++;
            t = tnext;
        }
        if (tnext >= tmax)
            break;
        i[ax] += st[ax];
        if (i[ax] < 0 || i[ax] >= n[ax])
            break;
    }
    return cnt <= cap ? cnt : -cnt;
}

int or_siddon_f64(const double o[3], const double d[3], const int32_t n[3], const double sp[3], int cap,
    int64_t* idx, double* len)
{
    double L[3], inv[3];
    double tmin = 0.0, tmax = DBL_MAX;
    for (int a = 0; a < 3; ++a) {
        L[a] = (double)n[a] * sp[a];
        if (d[a] != 0.0) {
            inv[a] = 1.0 / d[a];
            double t1 = (0.0 - o[a]) * inv[a];
            double t2 = (L[a] - o[a]) * inv[a];
            if (t1 > t2) {
                const double tt = t1;
                t1 = t2;
                t2 = tt;
            }
            if (t1 > tmin)
                tmin = t1;
            if (t2 < tmax)
                tmax = t2;
        } else {
            inv[a] = 0.0;
            if (o[a] < 0.0 || o[a] >= L[a])
                return 0;
        }
    }
    if (!(tmin < tmax))
        return 0;
    int i[3], st[3];
    for (int a = 0; a < 3; ++a) {
        const double p = o[a] + tmin * d[a];
        int k = (int)floor(p / sp[a]);
        if (k < 0)
            k = 0;
        if (k > n[a] - 1)
            k = n[a] - 1;
        i[a] = k;
        st[a] = d[a] > 0.0 ? 1 : (d[a] < 0.0 ? -1 : 0);
    }
    double t = tmin;
    int cnt = 0;
    for (;;) {
        double tn[3];
        for (int a = 0; a < 3; ++a)
            tn[a] = st[a] != 0 ? ((double)(i[a] + (st[a] > 0 ? 1 : 0)) * sp[a] - o[a]) * inv[a] : DBL_MAX;
        int ax = 0;
        if (tn[1] < tn[ax])
            ax = 1;
        if (tn[2] < tn[ax])
            ax = 2;
        double tnext = tn[ax] < tmax ? tn[ax] : tmax;
        const double l = tnext - t;
        if (l > 0.0) {
            if (cnt < cap) {
                idx[cnt] = (int64_t)i[0] + (int64_t)n[0] * ((int64_t)i[1] + (int64_t)n[1] * i[2]);
                len[cnt] = l;
            }
            cnt++;
            t = tnext;
        }
        if (tnext >= tmax)
            break;
        i[ax] += st[ax];
        if (i[ax] < 0 || i[ax] >= n[ax])
            break;
    }
    return cnt <= cap ? cnt : -cnt;
}

/* ------------------------------------------------------------------------- */
/* Material data for sampling: per element n_i = w_i / A_i (mol/g), Z_i, a_Z.  */
/* ------------------------------------------------------------------------- */
#define OR_MAX_SHELLS (3 * OR_MAX_ELEMENTS)
typedef struct {
    int n;
    double nZ[OR_MAX_ELEMENTS];  /* n_i Z_i   (incoherent scattering function weight) */
    double nZ2[OR_MAX_ELEMENTS]; /* n_i Z_i^2 (form-factor weight) */
    double a[OR_MAX_ELEMENTS];
    double Zsum;
    /* correction level 2 */
    double nZ4[OR_MAX_ELEMENTS]; /* n_i Z_i^4 (photoelectric share up to C / E^3) */
    double eK[OR_MAX_ELEMENTS], eL[OR_MAX_ELEMENTS], kAlpha[OR_MAX_ELEMENTS], omegaK[OR_MAX_ELEMENTS];
    int nShell;
    double shElectrons[OR_MAX_SHELLS], shBinding[OR_MAX_SHELLS], shMomentum[OR_MAX_SHELLS];
} mat_sampling;

static void make_sampling(const or_composition* c, mat_sampling* m)
{
    double w[OR_MAX_ELEMENTS];
    normalised(c, w);
    m->n = c->n;
    m->Zsum = 0.0;
    m->nShell = 0;
    for (int i = 0; i < c->n; ++i) {
        const double ni = w[i] / or_atomic_mass(c->Z[i]);
        m->nZ[i] = ni * c->Z[i];
        m->nZ2[i] = ni * c->Z[i] * c->Z[i];
        m->a[i] = a_Z(c->Z[i]);
        m->Zsum += m->nZ[i];
        const double z2 = (double)c->Z[i] * c->Z[i];
        m->nZ4[i] = ni * z2 * z2;
        m->eK[i] = or_k_edge(c->Z[i]);
        m->eL[i] = or_l_edge(c->Z[i]);
        m->kAlpha[i] = or_k_alpha(c->Z[i]);
        m->omegaK[i] = or_fluorescence_yield_k(c->Z[i]);
        double el[3], bd[3], mo[3];
        const int ns = or_compton_shells(c->Z[i], el, bd, mo);
        for (int k = 0; k < ns; ++k) {
            m->shElectrons[m->nShell] = ni * el[k];
            m->shBinding[m->nShell] = bd[k];
            m->shMomentum[m->nShell] = mo[k];
            m->nShell++;
        }
    }
}

/* Impulse-approximation energy for a projected electron momentum rho = p_z / m_e c
 * (Ribberfors 1975: rho = (E E' (1 - cos)/m_e c^2 - (E - E')) / |E - E'|, photon
 * momenta in keV), solved for E': with A = E / E_C and omu = 1 - cos,
 *   E'/E = (A - rho^2 cos + rho sqrt((A - cos)^2 + omu (2 - omu)(1 - rho^2))) / (A^2 - rho^2).
 * Returns 0 when no root exists. */
double or_doppler_energy(double E, double A, double omu, double rho)
{
    const double c = 1.0 - omu;
    const double den = A * A - rho * rho;
    const double disc = (A - c) * (A - c) + omu * (2.0 - omu) * (1.0 - rho * rho);
    if (!(den > 0.0) || !(disc >= 0.0))
        return 0.0;
    return E * ((A - rho * rho * c + rho * sqrt(disc)) / den);
}

/* Correction level 2 Compton energy: shell by its electrons among the shells bound
 * by less than E, projected momentum from the shell's profile
 * (1 + (p/p_s)^2)^-3 = Student-t with 5 degrees of freedom scaled by p_s / sqrt(5),
 * drawn by Bailey's polar method (Math. Comp. 62, 779, 1994); accepted when E' > 0
 * and E - E' exceeds the binding; 0 after DOPPLER_TRIES draws. */
#define DOPPLER_TRIES 32
static double doppler_sample(double E, double A, double omu, const mat_sampling* m, rng_t* r)
{
    double tot = 0.0;
    for (int k = 0; k < m->nShell; ++k)
        if (m->shBinding[k] < E)
            tot += m->shElectrons[k];
    const double target = rng_u(r) * tot;
    int sh = -1;
    double acc = 0.0;
    for (int k = 0; k < m->nShell; ++k) {
        if (m->shBinding[k] < E) {
            sh = k;
            acc += m->shElectrons[k];
            if (target <= acc)
                break;
        }
    }
    if (sh < 0)
        return 0.0;
    for (int t = 0; t < DOPPLER_TRIES; ++t) {
        const double a = 2.0 * rng_u(r) - 1.0;
        const double b = 2.0 * rng_u(r) - 1.0;
        const double w = a * a + b * b;
        if (w >= 1.0)
            continue;
        const double rho = m->shMomentum[sh] * a * sqrt((pow(w, -0.4) - 1.0) / w);
        const double e1 = or_doppler_energy(E, A, omu, rho);
        if (e1 > 0.0 && E - e1 > m->shBinding[sh])
            return e1;
    }
    return 0.0;
}

/* Correction level 2 photoelectric absorption: element by n_i Z_i^4 (/ J_K below its
 * K edge, / J_L below its L edge), K vacancy with probability 1 - 1/J_K above the
 * K edge, K-alpha emission with the yield omega_K.  Returns the fluorescence energy
 * or 0 (none above the cutoff). */
static double photo_share(double E, const mat_sampling* m, int i)
{
    double w = m->nZ4[i];
    if (E < m->eK[i])
        w /= J_K;
    if (E < m->eL[i])
        w /= J_L;
    return w;
}

static double sample_photo_fluorescence(double E, const mat_sampling* m, rng_t* r)
{
    double tot = 0.0;
    for (int i = 0; i < m->n; ++i)
        tot += photo_share(E, m, i);
    const double target = rng_u(r) * tot;
    int e = m->n - 1;
    double acc = 0.0;
    for (int i = 0; i < m->n; ++i) {
        acc += photo_share(E, m, i);
        if (target <= acc) {
            e = i;
            break;
        }
    }
    if (E < m->eK[e])
        return 0.0;
    if (rng_u(r) >= 1.0 - 1.0 / J_K)
        return 0.0;
    if (rng_u(r) >= m->omegaK[e])
        return 0.0;
    return m->kAlpha[e] >= E_CUT ? m->kAlpha[e] : 0.0;
}

static void isotropic_dir(double d[3], double u1, double u2)
{
    const double ct = 2.0 * u1 - 1.0;
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    const double phi = 2.0 * PI * u2;
    d[0] = st * cos(phi);
    d[1] = st * sin(phi);
    d[2] = ct;
}

/* Compton and Rayleigh angles (the transport kernel's samplers, jobs.cpp
 * comptonAngleRows / rayleighAngleRows and device.cuh): per table energy E_i, 1 - cos
 * theta at the cumulative probabilities u_j = (1 - cos(pi j/(K-1)))/2 of KN(mu) S(t(mu))
 * / Z (S = 1 at correction 0), or of (1 + mu^2)/2 F^2(x), integrated by the trapezoid rule
 * on 1024 equal steps of s with w = sqrt((1 - mu)/2) = s^2 and inverted linearly.  A draw
 * interpolates rows ie and ie + 1 at j = (K-1) acos(1 - 2u) / pi. */
#define OR_CTAB_K 256
static inline void grid_pos(double E, int* i, double* f);

/* One row of angle quantiles for a density f(1 - cos theta): trapezoid rule on G
 * equal steps of s with w = sqrt((1 - mu)/2) = s^P, inverted linearly. */
typedef double (*angle_density)(double omu, const void* ctx);

static void quantile_row(angle_density f, const void* ctx, int G, int P, double* row)
{
    double* cum = (double*)malloc((size_t)(G + 1) * sizeof(double));
    double prev = 0.0;
    for (int g = 0; g <= G; ++g) {
        const double sg = (double)g / G;
        const double w = P == 1 ? sg : sg * sg;
        const double dw = P == 1 ? 1.0 : 2.0 * sg;
        const double cur = f(2.0 * w * w, ctx) * 4.0 * w * dw;
        cum[g] = g == 0 ? 0.0 : cum[g - 1] + 0.5 * (prev + cur);
        prev = cur;
    }
    int g = 0;
    for (int j = OR_CTAB_K - 1; j >= 0; --j) {
        const double c = 0.5 * (1.0 + cos(PI * j / (OR_CTAB_K - 1))) * cum[G];
        while (g < G - 1 && cum[g + 1] < c)
            ++g;
        const double d = cum[g + 1] - cum[g];
        double fr = d > 0.0 ? (c - cum[g]) / d : 0.0;
        fr = fr < 0.0 ? 0.0 : (fr > 1.0 ? 1.0 : fr);
        const double sg = (g + fr) / G;
        const double w = P == 1 ? sg : sg * sg;
        row[j] = 2.0 * w * w;
    }
    row[0] = 2.0;
    row[OR_CTAB_K - 1] = 0.0;
    free(cum);
}

typedef struct {
    const mat_sampling* m;
    int correction;
    double k, q2;
} angle_ctx;

/* KN(mu) S(t(mu)) / Z, S = 1 at correction 0 */
static double compton_density(double omu, const void* c)
{
    const angle_ctx* x = (const angle_ctx*)c;
    const double mu = 1.0 - omu;
    const double P = 1.0 / (1.0 + x->k * omu);
    double f = P * P * (P + 1.0 / P - 1.0 + mu * mu);
    if (x->correction >= 1 && x->m->Zsum > 0.0) {
        const double t = x->q2 * 0.5 * omu;
        double S = 0.0;
        for (int e = 0; e < x->m->n; ++e) {
            const double b = 1.0 + t / x->m->a[e];
            const double b2 = b * b;
            S += x->m->nZ[e] * (1.0 - 1.0 / (b2 * b2));
        }
        f *= S / x->m->Zsum;
    }
    return f;
}

/* (1 + mu^2)/2 sum_i n_i Z_i^2 (1 + t/a_i)^-4 */
static double rayleigh_density(double omu, const void* c)
{
    const angle_ctx* x = (const angle_ctx*)c;
    const double mu = 1.0 - omu;
    const double t = x->q2 * 0.5 * omu;
    double F2 = 0.0;
    for (int e = 0; e < x->m->n; ++e) {
        const double b = 1.0 + t / x->m->a[e];
        const double b2 = b * b;
        F2 += x->m->nZ2[e] / (b2 * b2);
    }
    return 0.5 * (1.0 + mu * mu) * F2;
}

/* rows i0 .. i1 of a material's angle table: Compton (kind 0) or Rayleigh (kind 1) */
static void angle_rows(const mat_sampling* m, int kind, int correction, int i0, int i1, double* out)
{
    for (int i = i0; i <= i1; ++i) {
        const double E = OR_EMIN + i * OR_DE;
        angle_ctx x = { m, correction, E / ME_KEV, (E / HC_KEV_A) * (E / HC_KEV_A) };
        double* row = out + (size_t)(i - i0) * OR_CTAB_K;
        if (kind == 0)
            quantile_row(compton_density, &x, 1024, 2, row);
        else
            quantile_row(rayleigh_density, &x, 1024, 2, row);
    }
}

static void compton_rows(const mat_sampling* m, int correction, int i0, int i1, double* out)
{
    angle_rows(m, 0, correction, i0, i1, out);
}

/* 1 - cos theta from rows ie and ie + 1 of an angle table */
static double table_one_minus_cos(const double* rows, double fe, double u)
{
    const double jf = (OR_CTAB_K - 1) * acos(1.0 - 2.0 * u) / PI;
    int j = (int)jf;
    if (j > OR_CTAB_K - 2)
        j = OR_CTAB_K - 2;
    const double g = jf - j;
    const double lo = rows[j] + g * (rows[j + 1] - rows[j]);
    const double hi = rows[OR_CTAB_K + j] + g * (rows[OR_CTAB_K + j + 1] - rows[OR_CTAB_K + j]);
    return lo + fe * (hi - lo);
}

/* rows: the material's rows ie and ie + 1 (2 x OR_CTAB_K) */
static double sample_compton(double E, const mat_sampling* m, int correction, const double* rows, double fe,
    rng_t* r, double* cos_theta)
{
    const double k = E / ME_KEV;
    for (int guard = 0; guard < 100000; ++guard) {
        const double omu = table_one_minus_cos(rows, fe, rng_u(r)); /* 1 - cos theta */
        const double xm1 = k * omu;             /* x - 1, x = E / E' */
        *cos_theta = 1.0 - omu;
        if (correction >= 2) {
            const double Ep = doppler_sample(E, 1.0 + xm1, omu, m, r);
            if (Ep <= 0.0)
                continue;
            return Ep;
        }
        return E / (1.0 + xm1);
    }
    *cos_theta = 1.0;
    return E;
}

/* Rayleigh: cos theta from the material's quantile table of (1 + cos^2)/2 F^2(x)
 * (the transport kernel's sampler, jobs.cpp rayleighAngleRows and device.cuh
 * sampleRayleigh): rows ie and ie + 1, one uniform. */
static double sample_rayleigh(const double* rows, double fe, rng_t* r)
{
    return 1.0 - table_one_minus_cos(rows, fe, rng_u(r));
}

double or_sample_compton(double E, const or_composition* c, int correction, const double* u, int nu, int* used,
    double* cos_theta)
{
    mat_sampling m;
    make_sampling(c, &m);
    rng_t r;
    memset(&r, 0, sizeof(r));
    r.inj = u;
    r.n_inj = nu;
    int ie;
    double fe, rows[2 * OR_CTAB_K];
    grid_pos(E, &ie, &fe);
    compton_rows(&m, correction, ie, ie + 1, rows);
    const double Ep = sample_compton(E, &m, correction, rows, fe, &r, cos_theta);
    *used = r.used;
    return Ep;
}

int or_compton_quantiles(const or_composition* c, int correction, int energy_index, double* out)
{
    if (energy_index < 0 || energy_index >= OR_NE)
        return -1;
    mat_sampling m;
    make_sampling(c, &m);
    compton_rows(&m, correction, energy_index, energy_index, out);
    return OR_CTAB_K;
}

int or_rayleigh_quantiles(const or_composition* c, int energy_index, double* out)
{
    if (energy_index < 0 || energy_index >= OR_NE)
        return -1;
    mat_sampling m;
    make_sampling(c, &m);
    angle_rows(&m, 1, 0, energy_index, energy_index, out);
    return OR_CTAB_K;
}

double or_sample_photoelectric(double E, const or_composition* c, const double* u, int nu, int* used, double* dz)
{
    mat_sampling m;
    make_sampling(c, &m);
    rng_t r;
    memset(&r, 0, sizeof(r));
    r.inj = u;
    r.n_inj = nu;
    const double Ef = sample_photo_fluorescence(E, &m, &r);
    *dz = 0.0;
    if (Ef > 0.0) {
        double d[3];
        const double u1 = rng_u(&r);
        isotropic_dir(d, u1, rng_u(&r));
        *dz = d[2];
    }
    *used = r.used;
    return Ef;
}

double or_sample_rayleigh(double E, const or_composition* c, const double* u, int nu, int* used)
{
    mat_sampling m;
    make_sampling(c, &m);
    rng_t r;
    memset(&r, 0, sizeof(r));
    r.inj = u;
    r.n_inj = nu;
    int ie;
    double fe, rows[2 * OR_CTAB_K];
    grid_pos(E, &ie, &fe);
    angle_rows(&m, 1, 0, ie, ie + 1, rows);
    const double mu = sample_rayleigh(rows, fe, &r);
    *used = r.used;
    return mu;
}

/* ------------------------------------------------------------------------- */
/* World: AAVoxelGrid ingest + build (simulationpipeline.cpp:127-153).  Grid
 * centred on the origin (datacontainer.cpp:174-178), x fastest
 * (otherphantomimportpipeline.cpp:44), spacing in cm (datacontainer.cpp:241-253). */
/* ------------------------------------------------------------------------- */
struct or_world {
    int32_t n[3];
    double sp[3];
    size_t N;
    double* density;
    uint8_t* material;
    int n_mats;
    int correction;
    or_composition* mats;
    mat_sampling* samp;
    double* photo; /* [m][OR_NE] cm^2/g */
    double* incoh;
    double* coh;
    double* tot;
    double maj[OR_NE]; /* 1/cm */
    double* ctab;      /* [m][OR_NE][OR_CTAB_K] Compton 1 - cos theta quantiles */
    double* rtab;      /* [m][OR_NE][OR_CTAB_K] Rayleigh 1 - cos theta quantiles */
    /* two-region Woodcock: the box of voxels whose material is neither 0 nor
     * transparent (voxel indices b0 .. b1 inclusive), its faces widened by a margin,
     * and material 0's majorant; box_on 0: the box is empty or the whole grid */
    int box_on;
    int b0[3], b1[3];
    double blo[3], bhi[3];
    double maj_out[OR_NE];
    int mb;            /* macro-cell edge in voxels (0: none) */
    int mc[3];
    double* mscale;    /* per macro cell: majorant scale s_c */
    double* e;
    double* e2;
    uint64_t* cnt;
};

static const double MAJ_SAFETY = 1.0 + 1.0 / 1048576.0;

or_world* or_world_create(const int32_t dims[3], const double spacing_cm[3], const double* density,
    const uint8_t* material, const or_composition* mats, int n_mats, int correction)
{
    if (n_mats <= 0 || n_mats > 255)
        return NULL;
    or_world* w = (or_world*)calloc(1, sizeof(or_world));
    for (int a = 0; a < 3; ++a) {
        w->n[a] = dims[a];
        w->sp[a] = spacing_cm[a];
    }
    w->N = (size_t)dims[0] * dims[1] * dims[2];
    w->density = (double*)malloc(w->N * sizeof(double));
    w->material = (uint8_t*)malloc(w->N);
    memcpy(w->density, density, w->N * sizeof(double));
    memcpy(w->material, material, w->N);
    w->n_mats = n_mats;
    w->correction = correction;
    w->mats = (or_composition*)malloc(n_mats * sizeof(or_composition));
    memcpy(w->mats, mats, n_mats * sizeof(or_composition));
    w->samp = (mat_sampling*)malloc(n_mats * sizeof(mat_sampling));
    w->photo = (double*)malloc(n_mats * OR_NE * sizeof(double));
    w->incoh = (double*)malloc(n_mats * OR_NE * sizeof(double));
    w->coh = (double*)malloc(n_mats * OR_NE * sizeof(double));
    w->tot = (double*)malloc(n_mats * OR_NE * sizeof(double));
    double E[OR_NE];
    for (int i = 0; i < OR_NE; ++i)
        E[i] = OR_EMIN + i * OR_DE;
    w->ctab = (double*)malloc((size_t)n_mats * OR_NE * OR_CTAB_K * sizeof(double));
    w->rtab = (double*)malloc((size_t)n_mats * OR_NE * OR_CTAB_K * sizeof(double));
    for (int m = 0; m < n_mats; ++m) {
        make_sampling(&mats[m], &w->samp[m]);
        compton_rows(&w->samp[m], correction, 0, OR_NE - 1, w->ctab + (size_t)m * OR_NE * OR_CTAB_K);
        angle_rows(&w->samp[m], 1, 0, 0, OR_NE - 1, w->rtab + (size_t)m * OR_NE * OR_CTAB_K);
        or_attenuation(&mats[m], correction, OR_NE, E, w->photo + m * OR_NE, w->incoh + m * OR_NE,
            w->coh + m * OR_NE);
        for (int i = 0; i < OR_NE; ++i)
            w->tot[m * OR_NE + i] = w->photo[m * OR_NE + i] + w->incoh[m * OR_NE + i] + w->coh[m * OR_NE + i];
    }
    double rmax[256];
    for (int m = 0; m < 256; ++m)
        rmax[m] = 0.0;
    for (size_t v = 0; v < w->N; ++v) {
        const int m = w->material[v];
        if (m < n_mats && w->density[v] > rmax[m])
            rmax[m] = w->density[v];
    }
    for (int i = 0; i < OR_NE; ++i) {
        double mx = 0.0;
        for (int m = 0; m < n_mats; ++m) {
            const double v = rmax[m] * w->tot[m * OR_NE + i];
            if (v > mx)
                mx = v;
        }
        w->maj[i] = mx * MAJ_SAFETY;
        const double mo = rmax[0] * w->tot[i] * MAJ_SAFETY;
        w->maj_out[i] = mo > 1e-30 ? mo : 1e-30;
    }
    for (int a = 0; a < 3; ++a) {
        w->b0[a] = INT32_MAX;
        w->b1[a] = -1;
    }
    for (int z = 0; z < dims[2]; ++z)
        for (int y = 0; y < dims[1]; ++y)
            for (int x = 0; x < dims[0]; ++x) {
                const int m = w->material[(size_t)x + (size_t)dims[0] * ((size_t)y + (size_t)dims[1] * z)];
                if (m == 0 || m == OR_TRANSPARENT)
                    continue;
                const int i[3] = { x, y, z };
                for (int a = 0; a < 3; ++a) {
                    if (i[a] < w->b0[a])
                        w->b0[a] = i[a];
                    if (i[a] > w->b1[a])
                        w->b1[a] = i[a];
                }
            }
    w->box_on = w->b1[0] >= 0
        && (w->b0[0] > 0 || w->b0[1] > 0 || w->b0[2] > 0 || w->b1[0] < dims[0] - 1 || w->b1[1] < dims[1] - 1
            || w->b1[2] < dims[2] - 1);
    for (int a = 0; a < 3; ++a) {
        const double margin = 1e-3 * w->sp[a] > 1e-3 ? 1e-3 * w->sp[a] : 1e-3;
        w->blo[a] = w->b0[a] * w->sp[a] - margin;
        w->bhi[a] = (w->b1[a] + 1) * w->sp[a] + margin;
    }
    w->e = (double*)calloc(w->N, sizeof(double));
    w->e2 = (double*)calloc(w->N, sizeof(double));
    w->cnt = (uint64_t*)calloc(w->N, sizeof(uint64_t));
    return w;
}

void or_world_destroy(or_world* w)
{
    if (!w)
        return;
    free(w->density);
    free(w->material);
    free(w->mats);
    free(w->samp);
    free(w->photo);
    free(w->incoh);
    free(w->coh);
    free(w->tot);
    free(w->e);
    free(w->e2);
    free(w->cnt);
    free(w->mscale);
    free(w->ctab);
    free(w->rtab);
    free(w);
}

void or_world_clear(or_world* w)
{
    memset(w->e, 0, w->N * sizeof(double));
    memset(w->e2, 0, w->N * sizeof(double));
    memset(w->cnt, 0, w->N * sizeof(uint64_t));
}

int or_world_table(const or_world* w, int m, double* photo, double* incoh, double* coh)
{
    if (m < 0 || m >= w->n_mats)
        return -1;
    memcpy(photo, w->photo + m * OR_NE, OR_NE * sizeof(double));
    memcpy(incoh, w->incoh + m * OR_NE, OR_NE * sizeof(double));
    memcpy(coh, w->coh + m * OR_NE, OR_NE * sizeof(double));
    return OR_NE;
}

int or_world_majorant(const or_world* w, double* maj)
{
    memcpy(maj, w->maj, sizeof(w->maj));
    return OR_NE;
}

void or_world_tally(const or_world* w, double* energy, double* energy2, uint64_t* count)
{
    if (energy)
        memcpy(energy, w->e, w->N * sizeof(double));
    if (energy2)
        memcpy(energy2, w->e2, w->N * sizeof(double));
    if (count)
        memcpy(count, w->cnt, w->N * sizeof(uint64_t));
}

/* ------------------------------------------------------------------------- */
/* Transport                                                                   */
/* ------------------------------------------------------------------------- */
static inline void grid_pos(double E, int* i, double* f)
{
    const double x = (E - OR_EMIN) * (1.0 / OR_DE);
    int k = (int)x;
    if (k < 0)
        k = 0;
    if (k > OR_NE - 2)
        k = OR_NE - 2;
    *i = k;
    *f = x - k;
}

static inline double lerp_tab(const double* t, int i, double f) { return t[i] + f * (t[i + 1] - t[i]); }

static void atomic_add_f64(double* p, double v)
{
    uint64_t old = __atomic_load_n((uint64_t*)p, __ATOMIC_RELAXED);
    for (;;) {
        double cur;
        memcpy(&cur, &old, 8);
        const double nv = cur + v;
        uint64_t nb;
        memcpy(&nb, &nv, 8);
        if (__atomic_compare_exchange_n((uint64_t*)p, &old, nb, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED))
            return;
    }
}

typedef struct {
    int n;
    double E[512];
    uint32_t thr[512];
    int32_t alias[512];
} alias_table;

/* Walker alias table (Vose's O(n) construction). Acceptance thresholds are
 * stored as 23-bit integers so that the draw is exact on every device. */
static void build_alias(const double* w, int n, alias_table* t)
{
    double p[512];
    int small[512], large[512];
    int ns = 0, nl = 0;
    double s = 0.0;
    for (int i = 0; i < n; ++i)
        s += w[i];
    for (int i = 0; i < n; ++i) {
        p[i] = w[i] / s * n;
        t->alias[i] = i;
    }
    for (int i = 0; i < n; ++i) {
        if (p[i] < 1.0)
            small[ns++] = i;
        else
            large[nl++] = i;
    }
    double prob[512];
    while (ns > 0 && nl > 0) {
        const int l = small[--ns];
        const int g = large[--nl];
        prob[l] = p[l];
        t->alias[l] = g;
        p[g] = (p[g] + p[l]) - 1.0;
        if (p[g] < 1.0)
            small[ns++] = g;
        else
            large[nl++] = g;
    }
    while (nl > 0)
        prob[large[--nl]] = 1.0;
    while (ns > 0)
        prob[small[--ns]] = 1.0;
    for (int i = 0; i < n; ++i)
        t->thr[i] = (uint32_t)floor(prob[i] * 8388608.0 + 0.5);
    t->n = n;
}

static int sample_alias(const alias_table* t, rng_t* r)
{
    const uint32_t x0 = rng_raw(r) >> 9;
    const uint32_t x1 = rng_raw(r) >> 9;
    const int k = (int)(((uint64_t)x0 * (uint64_t)t->n) >> 23);
    return x1 < t->thr[k] ? k : t->alias[k];
}

typedef struct {
    int n;
    double ang[256];
    double w[256];
    double norm; /* mean over the tube's fan, |angle| in [0, half] */
} bowtie_t;

static double bowtie_eval(const bowtie_t* b, double a)
{
    if (b->n <= 0)
        return 1.0;
    if (a <= b->ang[0])
        return b->w[0];
    if (a >= b->ang[b->n - 1])
        return b->w[b->n - 1];
    int lo = 0, hi = b->n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (b->ang[mid] <= a)
            lo = mid;
        else
            hi = mid;
    }
    const double t = (a - b->ang[lo]) / (b->ang[hi] - b->ang[lo]);
    return b->w[lo] + t * (b->w[hi] - b->w[lo]);
}

/* mean of the bowtie profile over |angle| in [0, half] (exact for piecewise linear) */
static double bowtie_mean(const bowtie_t* b, double half)
{
    if (b->n <= 0 || half <= 0.0)
        return 1.0;
    double xs[260];
    int m = 0;
    xs[m++] = 0.0;
    for (int i = 0; i < b->n; ++i)
        if (b->ang[i] > 0.0 && b->ang[i] < half)
            xs[m++] = b->ang[i];
    xs[m++] = half;
    double s = 0.0;
    for (int i = 0; i + 1 < m; ++i)
        s += 0.5 * (bowtie_eval(b, xs[i]) + bowtie_eval(b, xs[i + 1])) * (xs[i + 1] - xs[i]);
    return s / half;
}

typedef struct {
    or_world* w;
    const or_beam* b;
    or_exposure* exps;
    int n_exp;
    double gorigin[3];
    alias_table spec[2];
    bowtie_t bow[2]; /* per tube: A, and dual-energy B */
    uint64_t seed;
    uint32_t stream;
    int tracking;
    uint64_t h0, h1;
    uint64_t next;
    pthread_mutex_t lock;
    or_stats tot;
} run_ctx;

static void deposit(or_world* w, size_t v, double e, or_stats* st)
{
    atomic_add_f64(&w->e[v], e);
    atomic_add_f64(&w->e2[v], e * e);
    __atomic_fetch_add(&w->cnt[v], 1, __ATOMIC_RELAXED);
    st->e_deposited += e;
    st->n_deposits++;
}

static void scatter_dir(double d[3], double cost, double phi_u)
{
    const double sint = sqrt(fmax(0.0, 1.0 - cost * cost));
    const double phi = 2.0 * PI * phi_u;
    const double cp = cos(phi), sp = sin(phi);
    double n[3];
    if (fabs(d[2]) > 0.99999) {
        n[0] = sint * cp;
        n[1] = sint * sp;
        n[2] = (d[2] > 0 ? 1.0 : -1.0) * cost;
    } else {
        const double tmp = sqrt(1.0 - d[2] * d[2]);
        n[0] = sint * (d[0] * d[2] * cp - d[1] * sp) / tmp + d[0] * cost;
        n[1] = sint * (d[1] * d[2] * cp + d[0] * sp) / tmp + d[1] * cost;
        n[2] = -sint * cp * tmp + d[2] * cost;
    }
    normalise3(n);
    d[0] = n[0];
    d[1] = n[1];
    d[2] = n[2];
}

static inline int inside(const or_world* w, const double p[3], size_t* v)
{
    int i[3];
    for (int a = 0; a < 3; ++a) {
        const double L = w->n[a] * w->sp[a];
        if (!(p[a] >= 0.0 && p[a] < L))
            return 0;
        int k = (int)floor(p[a] / w->sp[a]);
        if (k > w->n[a] - 1)
            k = w->n[a] - 1;
        i[a] = k;
    }
    *v = (size_t)i[0] + (size_t)w->n[0] * ((size_t)i[1] + (size_t)w->n[1] * i[2]);
    return 1;
}

/* Two-region Woodcock: voxel indices of p outside the box (p inside the grid). */
static inline int outside_box(const or_world* w, const double p[3])
{
    for (int a = 0; a < 3; ++a) {
        int k = (int)floor(p[a] / w->sp[a]);
        if (k > w->n[a] - 1)
            k = w->n[a] - 1;
        if (k < w->b0[a] || k > w->b1[a])
            return 1;
    }
    return 0;
}

/* Distance along d to the widened box (DBL_MAX if the line misses it, 0 from inside). */
static double box_entry(const or_world* w, const double p[3], const double d[3])
{
    double tn = 0.0, tf = DBL_MAX;
    for (int a = 0; a < 3; ++a) {
        if (d[a] == 0.0) {
            if (p[a] < w->blo[a] || p[a] > w->bhi[a])
                return DBL_MAX;
            continue;
        }
        double t1 = (w->blo[a] - p[a]) / d[a], t2 = (w->bhi[a] - p[a]) / d[a];
        if (t1 > t2) {
            const double tt = t1;
            t1 = t2;
            t2 = tt;
        }
        if (t1 > tn)
            tn = t1;
        if (t2 < tf)
            tf = t2;
    }
    return tn <= tf ? tn : DBL_MAX;
}

/* Real-interaction branch shared by both tracking modes; returns 0 if the photon died. */
static int interact(or_world* w, size_t v, int m, double* E, double wgt, double d[3], rng_t* r, or_stats* st,
    int* first)
{
    if (*first) {
        st->n_interacted++;
        *first = 0;
    }
    int ie;
    double fe;
    grid_pos(*E, &ie, &fe);
    const double ph = lerp_tab(w->photo + m * OR_NE, ie, fe);
    const double ic = lerp_tab(w->incoh + m * OR_NE, ie, fe);
    const double co = lerp_tab(w->coh + m * OR_NE, ie, fe);
    const double rt = rng_u(r) * (ph + ic + co);
    st->n_real++;
    if (rt < ph) {
        st->n_photo++;
        if (w->correction >= 2) {
            /* the atom may emit a K-alpha photon, followed from here in an isotropic direction */
            const double Ef = sample_photo_fluorescence(*E, &w->samp[m], r);
            deposit(w, v, wgt * (*E - Ef), st);
            if (Ef > 0.0) {
                st->n_fluorescence++;
                const double u1 = rng_u(r);
                isotropic_dir(d, u1, rng_u(r));
                *E = Ef;
                return 1;
            }
            return 0;
        }
        deposit(w, v, wgt * *E, st);
        return 0;
    }
    if (rt < ph + ic) {
        st->n_compton++;
        double cost;
        int ie;
        double fe;
        grid_pos(*E, &ie, &fe);
        const double Ep = sample_compton(*E, &w->samp[m], w->correction,
            w->ctab + ((size_t)m * OR_NE + ie) * OR_CTAB_K, fe, r, &cost);
        scatter_dir(d, cost, rng_u(r));
        deposit(w, v, wgt * (*E - Ep), st);
        *E = Ep;
        if (*E < E_CUT) {
            st->n_cutoff++;
            deposit(w, v, wgt * *E, st);
            return 0;
        }
        return 1;
    }
    st->n_rayleigh++;
    const double cost = sample_rayleigh(w->rtab + ((size_t)m * OR_NE + ie) * OR_CTAB_K, fe, r);
    scatter_dir(d, cost, rng_u(r));
    return 1;
}

/* Source photon of history h (draw order: 2 raw for the energy, fan, cone);
 * position in grid-local cm. */
static void sample_source(const run_ctx* c, uint64_t h, rng_t* r, double* E_out, double p[3], double d[3],
    double* wgt_out)
{
    const uint64_t ppe = c->b->particles_per_exposure;
    const or_exposure* ex = &c->exps[h / ppe];
    double E;
    if (c->b->type == OR_BEAM_PENCIL) {
        (void)rng_raw(r);
        (void)rng_raw(r);
        E = c->b->energy_kev;
    } else {
        const alias_table* at = &c->spec[ex->tube];
        E = at->E[sample_alias(at, r)];
    }
    const double ax = (2.0 * rng_u(r) - 1.0) * ex->half[0];
    const double ay = (2.0 * rng_u(r) - 1.0) * ex->half[1];
    const double sx = sin(ax), sy = sin(ay);
    const double sz = sqrt(fmax(0.0, 1.0 - sx * sx - sy * sy));
    double n[3];
    cross3(ex->c0, ex->c1, n);
    for (int a = 0; a < 3; ++a) {
        d[a] = ex->c0[a] * sx + ex->c1[a] * sy + n[a] * sz;
        p[a] = ex->pos[a] - c->gorigin[a];
    }
    double wgt = ex->weight;
    const bowtie_t* bow = &c->bow[ex->tube];
    if (bow->n > 0)
        wgt *= bowtie_eval(bow, fabs(ax)) / bow->norm;
    *E_out = E;
    *wgt_out = wgt;
}

static void run_history(run_ctx* c, uint64_t h, or_stats* st)
{
    or_world* w = c->w;
    rng_t r;
    rng_stream(&r, c->seed, c->stream, h);
    double E, wgt, p[3], d[3];
    sample_source(c, h, &r, &E, p, d, &wgt);
    int first = 1;
    st->n_histories++;
    st->e_source += wgt * E;
    /* enter the grid (slab test) */
    double tmin = 0.0, tmax = DBL_MAX;
    double L[3];
    for (int a = 0; a < 3; ++a) {
        L[a] = w->n[a] * w->sp[a];
        if (d[a] != 0.0) {
            double t1 = (0.0 - p[a]) / d[a], t2 = (L[a] - p[a]) / d[a];
            if (t1 > t2) {
                const double tt = t1;
                t1 = t2;
                t2 = tt;
            }
            if (t1 > tmin)
                tmin = t1;
            if (t2 < tmax)
                tmax = t2;
        } else if (p[a] < 0.0 || p[a] >= L[a]) {
            tmax = -1.0;
        }
    }
    if (!(tmin < tmax)) {
        st->n_missed++;
        st->e_escaped += wgt * E;
        return;
    }
    for (int a = 0; a < 3; ++a) {
        p[a] += tmin * d[a];
        if (p[a] < 0.0)
            p[a] = 0.0;
        if (p[a] >= L[a])
            p[a] = nextafter(L[a], 0.0);
    }
    /* two-region Woodcock: the flight starts against material 0's majorant when the
     * entry point lies outside the box */
    const int two = c->tracking == OR_TRACK_WOODCOCK_BOX && w->box_on;
    int outer = two && outside_box(w, p);
    int cell[3] = { 0, 0, 0 };
    if (c->tracking == OR_TRACK_MACRO) {
        if (!w->mscale) {
            st->n_errors++;
            return;
        }
        for (int a = 0; a < 3; ++a) {
            int k = (int)floor(p[a] / (w->mb * w->sp[a]));
            cell[a] = k < 0 ? 0 : (k > w->mc[a] - 1 ? w->mc[a] - 1 : k);
        }
    }
    for (long step = 0; step < MAX_STEPS; ++step) {
        if (c->tracking == OR_TRACK_MACRO) {
            /* delta tracking against the macro cell's majorant s_c * mu_max(E):
             * the sampled optical depth is spent cell by cell; a tentative collision
             * inside the cell is real with probability mu(voxel) / (s_c mu_max) */
            int ie;
            double fe;
            grid_pos(E, &ie, &fe);
            const double mmax = lerp_tab(w->maj, ie, fe);
            double tau = -log(rng_u(&r));
            for (;;) {
                const size_t ci = (size_t)cell[0] + (size_t)w->mc[0] * ((size_t)cell[1] + (size_t)w->mc[1] * cell[2]);
                const double muc = w->mscale[ci] * mmax;
                double tx = DBL_MAX;
                int ax = -1;
                for (int a = 0; a < 3; ++a) {
                    if (d[a] == 0.0)
                        continue;
                    double b = (cell[a] + (d[a] > 0.0 ? 1 : 0)) * w->mb * w->sp[a];
                    if (b > L[a])
                        b = L[a];
                    const double t = (b - p[a]) / d[a];
                    if (t < tx) {
                        tx = t;
                        ax = a;
                    }
                }
                if (tx < 0.0)
                    tx = 0.0;
                if (muc > 0.0 && tau < muc * tx) {
                    const double t = tau / muc;
                    for (int a = 0; a < 3; ++a)
                        p[a] += t * d[a];
                    break;
                }
                tau -= muc * tx;
                for (int a = 0; a < 3; ++a)
                    p[a] += tx * d[a];
                st->n_crossings++;
                cell[ax] += d[ax] > 0.0 ? 1 : -1;
                if (cell[ax] < 0 || cell[ax] >= w->mc[ax]) {
                    st->e_escaped += wgt * E;
                    return;
                }
            }
            /* voxel of the tentative collision, kept inside the current cell */
            int vi[3];
            for (int a = 0; a < 3; ++a) {
                int k = (int)floor(p[a] / w->sp[a]);
                const int lo = cell[a] * w->mb, hi = lo + w->mb - 1 < w->n[a] - 1 ? lo + w->mb - 1 : w->n[a] - 1;
                vi[a] = k < lo ? lo : (k > hi ? hi : k);
                if (p[a] < 0.0)
                    p[a] = 0.0;
                if (p[a] >= L[a])
                    p[a] = nextafter(L[a], 0.0);
            }
            const size_t v = (size_t)vi[0] + (size_t)w->n[0] * ((size_t)vi[1] + (size_t)w->n[1] * vi[2]);
            st->n_visits++;
            const int m = w->material[v];
            const size_t ci = (size_t)cell[0] + (size_t)w->mc[0] * ((size_t)cell[1] + (size_t)w->mc[1] * cell[2]);
            const double muc = w->mscale[ci] * mmax;
            if (m == OR_TRANSPARENT)
                continue;
            const double mu = w->density[v] * lerp_tab(w->tot + m * OR_NE, ie, fe);
            if (rng_u(&r) * muc < mu) {
                if (!interact(w, v, m, &E, wgt, d, &r, st, &first))
                    return;
            }
        } else if (c->tracking == OR_TRACK_WOODCOCK || c->tracking == OR_TRACK_WOODCOCK_BOX) {
            int ie;
            double fe;
            grid_pos(E, &ie, &fe);
            const double mmax = lerp_tab(outer ? w->maj_out : w->maj, ie, fe);
            const double s = -log(rng_u(&r)) / mmax;
            if (outer) {
                /* the box comes first: move there, no tentative collision */
                const double te = box_entry(w, p, d);
                if (te < s) {
                    for (int a = 0; a < 3; ++a)
                        p[a] += te * d[a];
                    outer = 0;
                    continue;
                }
            }
            for (int a = 0; a < 3; ++a)
                p[a] += s * d[a];
            size_t v;
            if (!inside(w, p, &v)) {
                st->e_escaped += wgt * E;
                return;
            }
            st->n_visits++;
            const int m = w->material[v];
            /* a flight against maj that ends outside the box: the flights after this
             * tentative collision step against material 0's majorant */
            const int leave = two && !outer && outside_box(w, p);
            int real = 0;
            if (m != OR_TRANSPARENT) {
                const double mu = w->density[v] * lerp_tab(w->tot + m * OR_NE, ie, fe);
                real = rng_u(&r) * mmax < mu;
            }
            if (leave)
                outer = 1;
            if (real) {
                /* a Rayleigh scattering keeps the flight's majorant; Compton scattering
                 * and fluorescence start again against maj */
                const uint64_t nr = st->n_rayleigh;
                if (!interact(w, v, m, &E, wgt, d, &r, st, &first))
                    return;
                if (st->n_rayleigh == nr)
                    outer = 0;
            }
        } else {
            /* regular tracking: walk voxel segments until the sampled optical depth is used up */
            const double tau = -log(rng_u(&r));
            int ie;
            double fe;
            grid_pos(E, &ie, &fe);
            int64_t idx[2048];
            double len[2048];
            const int32_t* nn = w->n;
            const int ns = or_siddon_f64(p, d, nn, w->sp, 2048, idx, len);
            double acc = 0.0, t = 0.0;
            int hit = -1;
            double thit = 0.0;
            for (int k = 0; k < (ns < 0 ? -ns : ns) && k < 2048; ++k) {
                st->n_visits++;
                const int m = w->material[idx[k]];
                const double mu = m == OR_TRANSPARENT ? 0.0 : w->density[idx[k]] * lerp_tab(w->tot + m * OR_NE, ie, fe);
                if (mu > 0.0 && acc + mu * len[k] >= tau) {
                    hit = k;
                    thit = t + (tau - acc) / mu;
                    break;
                }
                acc += mu * len[k];
                t += len[k];
            }
            if (hit < 0) {
                st->e_escaped += wgt * E;
                return;
            }
            for (int a = 0; a < 3; ++a) {
                p[a] += thit * d[a];
                if (p[a] < 0.0)
                    p[a] = 0.0;
                if (p[a] >= L[a])
                    p[a] = nextafter(L[a], 0.0);
            }
            const size_t v = (size_t)idx[hit];
            if (!interact(w, v, w->material[v], &E, wgt, d, &r, st, &first))
                return;
        }
    }
    st->n_errors++;
}

static void* worker(void* arg)
{
    run_ctx* c = (run_ctx*)arg;
    or_stats st;
    memset(&st, 0, sizeof(st));
    for (;;) {
        const uint64_t b = __atomic_fetch_add(&c->next, 4096, __ATOMIC_RELAXED);
        if (b >= c->h1)
            break;
        const uint64_t e = b + 4096 < c->h1 ? b + 4096 : c->h1;
        for (uint64_t h = b; h < e; ++h)
            run_history(c, h, &st);
    }
    pthread_mutex_lock(&c->lock);
    c->tot.e_source += st.e_source;
    c->tot.e_deposited += st.e_deposited;
    c->tot.e_escaped += st.e_escaped;
    c->tot.n_histories += st.n_histories;
    c->tot.n_missed += st.n_missed;
    c->tot.n_visits += st.n_visits;
    c->tot.n_real += st.n_real;
    c->tot.n_photo += st.n_photo;
    c->tot.n_compton += st.n_compton;
    c->tot.n_rayleigh += st.n_rayleigh;
    c->tot.n_deposits += st.n_deposits;
    c->tot.n_cutoff += st.n_cutoff;
    c->tot.n_errors += st.n_errors;
    c->tot.n_interacted += st.n_interacted;
    c->tot.n_crossings += st.n_crossings;
    c->tot.n_fluorescence += st.n_fluorescence;
    pthread_mutex_unlock(&c->lock);
    return NULL;
}

static int ctx_setup(run_ctx* c, or_world* w, const or_beam* b)
{
    memset(c, 0, sizeof(*c));
    c->w = w;
    c->b = b;
    c->n_exp = or_beam_exposures(b, NULL, 0);
    if (c->n_exp <= 0 || b->particles_per_exposure == 0)
        return -1;
    c->exps = (or_exposure*)malloc(c->n_exp * sizeof(or_exposure));
    or_beam_exposures(b, c->exps, c->n_exp);
    for (int a = 0; a < 3; ++a)
        c->gorigin[a] = -0.5 * w->n[a] * w->sp[a];
    if (b->type != OR_BEAM_PENCIL) {
        for (int t = 0; t < 2; ++t) {
            double E[512], wt[512];
            const int dual = b->type == OR_BEAM_CT_SPIRAL_DUAL && t == 1;
            const int n = or_tube_spectrum(dual ? b->kvp_b : b->kvp, b->anode_angle_deg,
                dual ? b->n_filters_b : b->n_filters, dual ? b->filter_Z_b : b->filter_Z,
                dual ? b->filter_mm_b : b->filter_mm, E, wt, 512);
            if (n <= 0) {
                if (t == 0) {
                    free(c->exps);
                    c->exps = NULL;
                    return -2;
                }
                c->spec[1] = c->spec[0];
                continue;
            }
            build_alias(wt, n, &c->spec[t]);
            memcpy(c->spec[t].E, E, n * sizeof(double));
        }
    }
    /* bowtie profiles: tube A from n_bowtie/bowtie_*, dual-energy tube B from
     * n_bowtie_b/bowtie_b_* (set independently, beamsettingsmodel.cpp:1581-1612) */
    for (int t = 0; t < 2; ++t) {
        bowtie_t* bw = &c->bow[t];
        bw->n = 0;
        bw->norm = 1.0;
        const int nb = t == 0 ? b->n_bowtie : (b->type == OR_BEAM_CT_SPIRAL_DUAL ? b->n_bowtie_b : 0);
        const double* ang = t == 0 ? b->bowtie_angle : b->bowtie_b_angle;
        const double* wt = t == 0 ? b->bowtie_weight : b->bowtie_b_weight;
        if (nb <= 0 || !ang || !wt)
            continue;
        /* sort by angle (the bowtie JSON is unordered, bowtiefilters.json:4-32) */
        const int n = nb > 256 ? 256 : nb;
        for (int i = 0; i < n; ++i) {
            bw->ang[i] = ang[i];
            bw->w[i] = wt[i];
        }
        for (int i = 1; i < n; ++i)
            for (int j = i; j > 0 && bw->ang[j - 1] > bw->ang[j]; --j) {
                double tmp = bw->ang[j];
                bw->ang[j] = bw->ang[j - 1];
                bw->ang[j - 1] = tmp;
                tmp = bw->w[j];
                bw->w[j] = bw->w[j - 1];
                bw->w[j - 1] = tmp;
            }
        bw->n = n;
        double half = 0.0;
        for (int i = 0; i < c->n_exp; ++i)
            if (c->exps[i].tube == t) {
                half = c->exps[i].half[0];
                break;
            }
        bw->norm = bowtie_mean(bw, half);
    }
    return 0;
}

int or_transport(or_world* w, const or_beam* b, uint64_t seed, uint32_t stream, int tracking, int n_threads,
    uint64_t hist_begin, uint64_t hist_end, or_stats* stats)
{
    run_ctx c;
    const int rc = ctx_setup(&c, w, b);
    if (rc != 0)
        return rc;
    c.seed = seed;
    c.stream = stream;
    c.tracking = tracking;
    const uint64_t total = (uint64_t)c.n_exp * b->particles_per_exposure;
    c.h0 = hist_begin;
    c.h1 = hist_end < total ? hist_end : total;
    c.next = c.h0;
    pthread_mutex_init(&c.lock, NULL);
    if (n_threads < 1)
        n_threads = 1;
    pthread_t* th = (pthread_t*)malloc(n_threads * sizeof(pthread_t));
    for (int i = 0; i < n_threads; ++i)
        pthread_create(&th[i], NULL, worker, &c);
    for (int i = 0; i < n_threads; ++i)
        pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&c.lock);
    free(c.exps);
    if (stats)
        *stats = c.tot;
    return 0;
}

int or_sample_source(or_world* w, const or_beam* b, uint64_t seed, uint32_t stream, uint64_t h0, int n, double* out8)
{
    run_ctx c;
    const int rc = ctx_setup(&c, w, b);
    if (rc != 0)
        return rc;
    for (int i = 0; i < n; ++i) {
        rng_t r;
        rng_stream(&r, seed, stream, h0 + i);
        double E, wgt, p[3], d[3];
        sample_source(&c, h0 + i, &r, &E, p, d, &wgt);
        double* o = out8 + 8 * (size_t)i;
        o[0] = E;
        o[1] = wgt;
        o[2] = p[0];
        o[3] = p[1];
        o[4] = p[2];
        o[5] = d[0];
        o[6] = d[1];
        o[7] = d[2];
    }
    free(c.exps);
    return 0;
}

void or_history_stream(uint64_t seed, uint32_t stream, uint64_t h0, int n_hist, int n_draws, uint32_t* out)
{
    for (int i = 0; i < n_hist; ++i) {
        rng_t r;
        rng_stream(&r, seed, stream, h0 + (uint64_t)i);
        for (int k = 0; k < n_draws; ++k)
            out[(size_t)i * n_draws + k] = rng_raw(&r);
    }
}

/* Macro cells of B x B x B voxels.  s_c bounds mu(voxel, E) / mu_max(E) over the cell
 * for every table energy: s_c = max over its voxels of rho * r_m (times a small
 * safety factor), r_m = max_E mu_m(E) / mu_max(E). */
int or_world_set_macro(or_world* w, int B, double* scale_out)
{
    if (B < 1)
        return -1;
    double r[256];
    for (int m = 0; m < w->n_mats; ++m) {
        double mx = 0.0;
        for (int i = 0; i < OR_NE; ++i)
            if (w->maj[i] > 0.0) {
                const double q = w->tot[m * OR_NE + i] / w->maj[i];
                if (q > mx)
                    mx = q;
            }
        r[m] = mx;
    }
    free(w->mscale);
    w->mb = B;
    for (int a = 0; a < 3; ++a)
        w->mc[a] = (w->n[a] + B - 1) / B;
    const size_t nc = (size_t)w->mc[0] * w->mc[1] * w->mc[2];
    w->mscale = (double*)calloc(nc, sizeof(double));
    for (int k = 0; k < w->n[2]; ++k)
        for (int j = 0; j < w->n[1]; ++j)
            for (int i = 0; i < w->n[0]; ++i) {
                const size_t v = (size_t)i + (size_t)w->n[0] * ((size_t)j + (size_t)w->n[1] * k);
                const int m = w->material[v];
                if (m >= w->n_mats)
                    continue;
                const double s = w->density[v] * r[m] * MAJ_SAFETY;
                const size_t c = (size_t)(i / B) + (size_t)w->mc[0] * ((size_t)(j / B) + (size_t)w->mc[1] * (k / B));
                if (s > w->mscale[c])
                    w->mscale[c] = s;
            }
    if (scale_out)
        memcpy(scale_out, w->mscale, nc * sizeof(double));
    return (int)nc;
}
