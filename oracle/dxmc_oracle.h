/*
 * dxmc_oracle.h -- CPU oracle for the photon-transport hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker, never the product: only the
 * test-suite, the smoke check and the benchmark's CPU-baseline leg load it.
 *
 * It restates, in plain C with FP64 arithmetic, the path OpenDXMC reaches at
 * src/libopendxmc/simulationpipeline.cpp:165 (`transport(world, beam, progress, true)`):
 * world ingest (simulationpipeline.cpp:127-153), tube spectrum
 * (ctsegmentationpipeline.cpp:66-71), beam -> exposures (dxmc_specialization.cpp:78-90,
 * beamactorcontainer.cpp:44-67, :110-170), per-history source sampling, voxel traversal,
 * interaction sampling and per-voxel energy scoring (readback at
 * simulationpipeline.cpp:174-231).
 *
 * PARITY UNPINNED: the arithmetic of that call lives in DXMClib, which is not part
 * of the reference tree (CMakeLists.txt:68-75 fetches branch `develop`, no pinned
 * commit) and ships no known-answer tests.  The oracle therefore restates the
 * algorithm from the call sites, with a project-authored parametric physics model
 * (documented in physics comments below), and is pinned against analytic known
 * answers (Klein-Nishina integrals, Beer-Lambert transmission, energy
 * conservation) and the reference's own data files (media.dat, bowtie JSON).
 */
#ifndef DXMC_ORACLE_H
#define DXMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Energy grid of the attenuation tables: E_i = OR_EMIN + i * OR_DE keV. */
#define OR_NE 300
#define OR_EMIN 1.0
#define OR_DE 0.5
#define OR_MAX_ELEMENTS 16
#define OR_TRANSPARENT 255

/* OR_TRACK_WOODCOCK_BOX: Woodcock with two regions, the transport kernel's default
 * (outside the box of voxels whose material is neither 0 nor transparent, flights
 * step against material 0's majorant until they reach the box) */
enum { OR_TRACK_WOODCOCK = 0, OR_TRACK_SIDDON = 1, OR_TRACK_MACRO = 2, OR_TRACK_WOODCOCK_BOX = 3 };
enum {
    OR_BEAM_DX = 0,
    OR_BEAM_CT_SPIRAL = 1,
    OR_BEAM_CT_SEQUENTIAL = 2,
    OR_BEAM_CBCT = 3,
    OR_BEAM_PENCIL = 4,
    OR_BEAM_CT_SPIRAL_DUAL = 5
};

typedef struct {
    int32_t n;
    int32_t Z[OR_MAX_ELEMENTS];
    double w[OR_MAX_ELEMENTS]; /* mass fractions, normalised on use */
} or_composition;

/* Beam parameters, the union of what the OpenDXMC beam setters carry
 * (beamsettingsmodel.cpp:459-1837).  Geometry is in world cm, angles in radians
 * unless the field name says deg. */
typedef struct {
    int32_t type;
    double kvp;
    double anode_angle_deg;
    int32_t n_filters;
    int32_t filter_Z[8];
    double filter_mm[8];
    uint64_t particles_per_exposure;
    uint64_t n_exposures; /* DX / pencil: number of identical exposures ("jobs") */
    /* DX, pencil, CT sequential */
    double position[3];
    double cosines[2][3];
    double half_angles[2];
    double energy_kev; /* pencil beam mono-energy */
    /* CT */
    double start[3];
    double stop[3];
    double start_angle_deg;
    double stop_angle_deg;
    double step_angle_deg;
    double pitch;
    double collimation_cm;
    double scan_fov_cm;
    double sdd_cm;
    double rotation_axis[3];
    int32_t n_slices; /* CT sequential: number of axial positions */
    double slice_spacing_cm;
    double kvp_b; /* dual energy: second tube */
    int32_t n_filters_b;
    int32_t filter_Z_b[8];
    double filter_mm_b[8];
    double tube_a_weight; /* dual energy: relative mAs of tube A */
    double fov_b_cm;
    /* bowtie (angle rad, weight), unsorted allowed */
    int32_t n_bowtie;
    const double* bowtie_angle;
    const double* bowtie_weight;
    /* AEC (CTAECFilter(start, stop, weights)) */
    int32_t n_aec;
    double aec_start[3];
    double aec_stop[3];
    const double* aec_weight;
    /* organ AEC: lowered tube output over an angular sector (beamsettingsmodel.cpp:349-438) */
    int32_t organ_aec;
    double organ_aec_start_deg;
    double organ_aec_stop_deg;
    double organ_aec_ramp_deg;
    double organ_aec_low_weight;
    int32_t organ_aec_compensate;
    /* calibration targets (not used by the oracle's transport) */
    double dap_mgycm2;
    double ctdi_vol_mgy;
    double ctdi_w_mgy;
    double ctdi_diameter_cm;
    double air_kerma_mgy; /* pencil beam: air kerma of one history per cm2 */
    /* dual energy: tube B's bowtie (the fields above are tube A's); 0 points: none */
    int32_t n_bowtie_b;
    const double* bowtie_b_angle;
    const double* bowtie_b_weight;
} or_beam;

typedef struct {
    double pos[3]; /* world cm */
    double c0[3];
    double c1[3];
    double half[2];
    double weight;
    int32_t tube; /* 0 = A, 1 = B (dual energy) */
} or_exposure;

typedef struct {
    double e_source, e_deposited, e_escaped;
    uint64_t n_histories, n_missed, n_visits, n_real, n_photo, n_compton, n_rayleigh,
        n_deposits, n_cutoff, n_errors, n_interacted, n_crossings, n_fluorescence;
} or_stats;

typedef struct or_world or_world;

/* physics tables ("dxmcg-physics 1" text, as the engine reads it): load replaces the
 * model's numbers for the listed elements and tube settings (0, or < 0 on a bad
 * file, which leaves the model alone); reset returns to the model */
int or_physics_load(const char* path);
void or_physics_reset(void);
/* physics (per atom, barn; energies keV) */
double or_atomic_mass(int Z);
double or_element_density(int Z);
double or_sigma_kn(double E);
double or_sigma_photo(double E, int Z);
double or_sigma_incoh(double E, int Z, int correction);
double or_sigma_coh(double E, int Z);
double or_kn_energy_transfer_fraction(double E);
/* mass coefficients (cm^2/g) of a composition at arbitrary energies */
void or_attenuation(const or_composition* c, int correction, int n, const double* E,
    double* photo, double* incoh, double* coh);
/* tube */
int or_tube_spectrum(double kvp, double anode_angle_deg, int n_filters, const int32_t* fZ,
    const double* fmm, double* energies, double* weights, int cap);
double or_tube_mean_energy(double kvp, int n_filters, const int32_t* fZ, const double* fmm);
double or_tube_al_hvl_mm(double kvp, int n_filters, const int32_t* fZ, const double* fmm);
/* rng */
double or_uniform_from_u32(uint32_t x);
/* raw draws of the per-history streams (xoshiro128+ seeded by SplitMix64) */
void or_history_stream(uint64_t seed, uint32_t stream, uint64_t h0, int n_hist, int n_draws, uint32_t* out);
/* beam geometry */
int or_beam_exposures(const or_beam* b, or_exposure* out, int cap);
/* analytic calibration factor over n_hist histories: DX/CBCT (DAP), pencil (air
 * kerma); 1 without a target, -1 for CT beams */
double or_calibration_factor(const or_beam* b, uint64_t n_hist);
/* traversal on a grid-local ray; returns number of segments (or -needed if cap too small) */
int or_siddon_f32(const float o[3], const float d[3], const int32_t n[3], const float sp[3], int cap,
    int64_t* idx, float* len);
int or_siddon_f64(const double o[3], const double d[3], const int32_t n[3], const double sp[3], int cap,
    int64_t* idx, double* len);
/* samplers driven by injected uniforms (u consumed sequentially, *used returns count) */
double or_sample_compton(double E, const or_composition* c, int correction, const double* u,
    int nu, int* used, double* cos_theta);
double or_sample_rayleigh(double E, const or_composition* c, const double* u, int nu, int* used);
/* correction level 2 photoelectric absorption: fluorescence energy (0: none), dz of its direction */
double or_sample_photoelectric(double E, const or_composition* c, const double* u, int nu, int* used, double* dz);
/* correction level 2 element data and the impulse-approximation energy relation */
double or_k_edge(int Z);
double or_l_edge(int Z);
double or_k_alpha(int Z);
double or_fluorescence_yield_k(int Z);
int or_compton_shells(int Z, double electrons[3], double binding[3], double momentum[3]);
double or_doppler_energy(double E, double A, double omu, double rho);
/* world */
or_world* or_world_create(const int32_t dims[3], const double spacing_cm[3], const double* density,
    const uint8_t* material, const or_composition* mats, int n_mats, int correction);
void or_world_destroy(or_world* w);
void or_world_clear(or_world* w);
int or_world_table(const or_world* w, int m, double* photo, double* incoh, double* coh);
int or_world_majorant(const or_world* w, double* maj);
/* macro cells of B^3 voxels with majorant scales (for OR_TRACK_MACRO); fills scale if not NULL */
int or_world_set_macro(or_world* w, int B, double* scale_out);
/* Compton angle table row: 1 - cos theta at u_j = 1 - (1 - j/(K-1))^2, j < K (returns
 * K = 256), for table energy OR_EMIN + energy_index * OR_DE */
int or_compton_quantiles(const or_composition* c, int correction, int energy_index, double* out);
/* the same for the Rayleigh angle, (1 + cos^2)/2 F^2(x) */
int or_rayleigh_quantiles(const or_composition* c, int energy_index, double* out);
int or_transport(or_world* w, const or_beam* b, uint64_t seed, uint32_t stream, int tracking,
    int n_threads, uint64_t hist_begin, uint64_t hist_end, or_stats* stats);
int or_sample_source(or_world* w, const or_beam* b, uint64_t seed, uint32_t stream, uint64_t h0, int n,
    double* out8);
void or_world_tally(const or_world* w, double* energy, double* energy2, uint64_t* count);

#ifdef __cplusplus
}
#endif
#endif
