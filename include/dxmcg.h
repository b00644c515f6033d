/*
 * dxmcg.h -- C ABI of the GB300 photon-transport engine (libdxmcg.so).
 *
 * This is the drop-in boundary for the one call OpenDXMC makes into DXMClib's
 * Monte Carlo engine:
 *
 *     transport(world, beam, progress, true);      src/libopendxmc/simulationpipeline.cpp:165
 *
 * together with the world ingest before it (simulationpipeline.cpp:127-153) and
 * the per-voxel readback after it (simulationpipeline.cpp:174-231).  Plain C types
 * only: pointers, sizes, status codes.  No exceptions cross this boundary.  The
 * header-only C++ shim under include/dxmc/ re-creates the dxmc:: classes OpenDXMC
 * compiles against on top of these functions.
 *
 * Conventions
 *  - lengths in cm, energies in keV, angles in radians unless a name says _deg;
 *  - voxel index i + nx*(j + ny*k), x fastest (otherphantomimportpipeline.cpp:44);
 *  - the grid is centred on the world origin (datacontainer.cpp:174-178);
 *  - every function returns DXMCG_OK (0) or a negative dxmcg_status; the text of
 *    the last error on the calling thread is returned by dxmcg_last_error().
 */
#ifndef DXMCG_H
#define DXMCG_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define DXMCG_API __attribute__((visibility("default")))
#else
#define DXMCG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define DXMCG_VERSION 1
#define DXMCG_MAX_ELEMENTS 16
#define DXMCG_MAX_MATERIALS 255
#define DXMCG_TRANSPARENT_MATERIAL 255
#define DXMCG_NE 300 /* attenuation table energies: 1.0 + 0.5 i keV */

typedef enum {
    DXMCG_OK = 0,
    DXMCG_ERR_ARGUMENT = -1,
    DXMCG_ERR_CUDA = -2,
    DXMCG_ERR_STATE = -3,
    DXMCG_ERR_CANCELLED = -4,
    DXMCG_ERR_DEVICE = -5, /* a device-side check failed (step limit, bad voxel) */
    DXMCG_ERR_NO_DEVICE = -6,
    DXMCG_ERR_CAPACITY = -7
} dxmcg_status;

typedef enum {
    DXMCG_BEAM_DX = 0,
    DXMCG_BEAM_CT_SPIRAL = 1,
    DXMCG_BEAM_CT_SEQUENTIAL = 2,
    DXMCG_BEAM_CBCT = 3,
    DXMCG_BEAM_PENCIL = 4,
    DXMCG_BEAM_CT_SPIRAL_DUAL_ENERGY = 5
} dxmcg_beam_type;

/* WOODCOCK: delta tracking against the grid-wide majorant mu_max(E).
 * SIDDON: regular tracking with exact voxel path lengths.
 * MACRO: delta tracking against a per-macro-cell majorant s_c mu_max(E), cells of
 *        macro_cell^3 voxels; the sampled optical depth is spent cell by cell. */
typedef enum { DXMCG_TRACK_WOODCOCK = 0, DXMCG_TRACK_SIDDON = 1, DXMCG_TRACK_MACRO = 2 } dxmcg_tracking;

/* Material by mass fractions of elements: Material<5>::byWeight(map<Z, w>)
 * (simulationpipeline.cpp:136). Weights are normalised by the library. */
typedef struct {
    int32_t n;
    int32_t Z[DXMCG_MAX_ELEMENTS];
    double w[DXMCG_MAX_ELEMENTS];
} dxmcg_material;

/* Union of the beam parameters the OpenDXMC beam setters carry
 * (beamsettingsmodel.cpp:459-1837; dxmc_specialization.hpp:37-77). */
typedef struct {
    int32_t type; /* dxmcg_beam_type */
    double kvp;   /* setTubeVoltage (beamsettingsmodel.cpp:262) */
    double anode_angle_deg;
    int32_t n_filters; /* addTubeFiltrationMaterial(Z, mm) (beamsettingsmodel.cpp:286-323) */
    int32_t filter_Z[8];
    double filter_mm[8];
    uint64_t particles_per_exposure;
    uint64_t n_exposures; /* DX / pencil: number of identical exposures */
    /* DX, pencil, CT sequential */
    double position[3];
    double cosines[2][3]; /* direction cosines; beam direction = c0 x c1 */
    double half_angles[2]; /* collimation half angles */
    double energy_kev;     /* pencil beam */
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
    int32_t n_slices;
    double slice_spacing_cm;
    double kvp_b; /* dual energy, tube B */
    int32_t n_filters_b;
    int32_t filter_Z_b[8];
    double filter_mm_b[8];
    double tube_a_weight;
    double fov_b_cm;
    /* bowtie (BowtieFilter(vector<pair<angle_rad, weight>>), bowtiefilterreader.cpp:64-92) */
    int32_t n_bowtie;
    const double* bowtie_angle;
    const double* bowtie_weight;
    /* AEC (CTAECFilter(start, stop, weights), datacontainer.cpp:53-62) */
    int32_t n_aec;
    double aec_start[3];
    double aec_stop[3];
    const double* aec_weight;
    /* organ AEC: tube output lowered over an angular sector (beamsettingsmodel.cpp:349-438) */
    int32_t organ_aec;
    double organ_aec_start_deg;
    double organ_aec_stop_deg;
    double organ_aec_ramp_deg;
    double organ_aec_low_weight;
    int32_t organ_aec_compensate;
    /* dose calibration targets used when dxmcg_run_options.normalize is set:
     * DX / CBCT: dose-area product (setDAPvalue, beamsettingsmodel.cpp:576);
     * CT: CTDIvol, or CTDIw when ctdi_vol_mgy is 0, measured in a PMMA phantom of
     * ctdi_diameter_cm (setCTDIvol / setCTDIw / setCTDIdiameter, :1054, :1278-1293) */
    double dap_mgycm2;
    double ctdi_vol_mgy;
    double ctdi_w_mgy;
    double ctdi_diameter_cm;
    /* pencil beam calibration target: air kerma (mGy) of one history per cm2
     * (PencilBeam::setAirKerma, beamsettingsmodel.cpp:675) */
    double air_kerma_mgy;
    /* dual energy: tube B's bowtie (setBowtieFilterB, beamsettingsmodel.cpp:1607-1612);
     * n_bowtie/bowtie_angle/bowtie_weight above are tube A's.  n_bowtie_b = 0: no
     * bowtie on tube B.  Ignored by the single-tube beams. */
    int32_t n_bowtie_b;
    const double* bowtie_b_angle;
    const double* bowtie_b_weight;
} dxmcg_beam;

/* One source pose (exposure(i) in beamactorcontainer.cpp:114-121). */
typedef struct {
    double pos[3];
    double c0[3];
    double c1[3];
    double half[2];
    double weight;
    int32_t tube;
} dxmcg_exposure;

typedef struct {
    uint64_t seed;        /* random streams: seed */
    uint32_t stream;      /* stream word: independent streams per beam or per replica */
    int32_t tracking;     /* dxmcg_tracking */
    int32_t normalize;    /* trailing bool of transport(...): scale dose to the beam's DAP */
    int32_t block_size;   /* 0 = library default / autotuned */
    int32_t blocks_per_sm;
    int32_t chunk_histories_log2; /* histories per launch (progress/cancel granularity), 0 = default */
    uint64_t hist_begin;  /* history range [begin, end) of the beam; end 0 = all */
    uint64_t hist_end;
    int32_t interact_batch; /* parked scatterings a warp gathers before sampling them, 0 = default */
    int32_t refill_batch;   /* dead lanes a warp gathers before starting new histories, 0 = default */
    int32_t macro_cell;     /* MACRO tracking: cell edge in voxels, 0 = default (16) */
    int32_t woodcock_steps; /* WOODCOCK tracking: steps a lane takes between regroupings, 0 = default:
                             * 1.4 / p clamped to 4..16, p = stops per step of the world's
                             * previous Woodcock run (8 before the first) */
    /* per-history step limit, 0 = default (1,000,000, at most that): a history that
     * takes more tracking steps is stopped and counted in n_errors, and the call
     * returns DXMCG_ERR_DEVICE after the launch completes */
    uint32_t max_steps;
    /* WOODCOCK tracking, gather skip: a tentative collision whose 8x8x8-voxel cell
     * bound already proves it virtual does not read its voxel (the same decisions,
     * fewer voxel reads).  1 = on, -1 = off, 0 = default: on when the voxel words
     * (4 bytes per voxel; for a batch, of all its worlds, decided from opts[0])
     * exceed 64 MiB, where they no longer stay in L2 */
    int32_t gather_skip;
    /* WOODCOCK tracking, two regions: outside the bounding box of the voxels whose
     * material is neither 0 nor transparent, flights step against material 0's own
     * majorant until they reach the box (the same transport, fewer tentative
     * collisions in the air around a patient).  1 = on, -1 = off, 0 = default: on
     * when that box holds less than half of the grid's voxels (decided per world,
     * also in a batch) */
    int32_t two_region;
} dxmcg_run_options;

typedef struct {
    double e_source, e_deposited, e_escaped; /* keV, weighted */
    uint64_t n_histories, n_missed, n_visits, n_photo, n_compton, n_rayleigh, n_cutoff, n_errors;
    uint64_t n_interacted; /* histories with at least one real interaction */
    double kernel_ms;   /* device time of the transport launches (CUDA events) */
    double total_ms;    /* host wall time of the call */
    double dose_scale;  /* mGy per (keV / g) applied by the dose readout */
    double calibration; /* factor applied to every history weight (1 unless normalize) */
    uint64_t n_crossings; /* MACRO tracking: macro-cell boundary crossings */
    uint64_t n_fluorescence; /* correction level 2: K fluorescence photons emitted */
    uint64_t n_voxel_reads;  /* voxel words read: n_visits less the tentative collisions
                                the Woodcock gather skip settled from their cell bound */
    uint64_t n_cell_reads;   /* gather-skip cell bounds read (the tentative collisions inside
                                the two-region box when the skip ran) */
    int32_t woodcock_steps;  /* WOODCOCK tracking: steps per phase the launches used */
    int32_t two_region;      /* WOODCOCK tracking: 1 when the run used two regions */
} dxmcg_stats;

typedef struct dxmcg_world dxmcg_world;
typedef struct dxmcg_progress dxmcg_progress;

DXMCG_API int dxmcg_version(void);
DXMCG_API const char* dxmcg_last_error(void);
/* number of CUDA devices; 0 when none */
DXMCG_API int dxmcg_device_count(void);
/* device that later dxmcg_world_create calls on this thread use (one process per GPU) */
DXMCG_API int dxmcg_set_device(int device);

/* ---- host physics (FP64): Material<5>::attenuationValues, Tube --------------
 * (ctsegmentationpipeline.cpp:66-104)                                        */
DXMCG_API int dxmcg_material_attenuation(const dxmcg_material* m, int correction, int n, const double* energies,
    double* photo, double* incoherent, double* coherent);
DXMCG_API int dxmcg_tube_spectrum(double kvp, double anode_angle_deg, int n_filters, const int32_t* filter_Z,
    const double* filter_mm, double* energies, double* weights, int cap, int* n_out);
DXMCG_API int dxmcg_tube_mean_energy(double kvp, int n_filters, const int32_t* filter_Z, const double* filter_mm,
    double* mean_kev);
DXMCG_API int dxmcg_tube_al_hvl(double kvp, int n_filters, const int32_t* filter_Z, const double* filter_mm,
    double* hvl_mm);
/* ---- physics tables --------------------------------------------------------
 * The interaction data behind Material<5>::byWeight (simulationpipeline.cpp:136)
 * and the Tube (ctsegmentationpipeline.cpp:66-71).  The engine's own model is
 * parametric; a table file (text, "dxmcg-physics 1": an energy grid, then per
 * element its atomic mass, photoelectric, incoherent and coherent cross sections
 * in barn/atom on that grid, form-factor scale, K/L edges, K-alpha energy and
 * yield, and Compton shells; optionally unfiltered tube spectra per kVp and anode
 * angle) replaces those numbers for the elements and tubes it lists.  The format
 * is described in full in opendxmc_gb300/csrc/physics.hpp.  Process-wide; worlds
 * built and spectra made after a load use it.  write dumps the current numbers of
 * the listed elements on the DXMCG_NE-point table grid (loading that file back
 * leaves every device table bit for bit as it was). */
DXMCG_API int dxmcg_physics_load(const char* path);
DXMCG_API int dxmcg_physics_reset(void);
DXMCG_API int dxmcg_physics_write(const char* path, int n_elements, const int32_t* Z);
/* numberOfExposures()/exposure(i) (beamactorcontainer.cpp:114-121); out may be NULL to count */
DXMCG_API int dxmcg_beam_exposures(const dxmcg_beam* beam, dxmcg_exposure* out, int cap, int* n_out);
/* The factor dxmcg_transport_run applies to every history weight when
 * opts->normalize is set (the trailing `true` of transport(...),
 * simulationpipeline.cpp:165), referred to all N = exposures x
 * particles_per_exposure histories of the beam: DX/CBCT from dap_mgycm2, pencil
 * from air_kerma_mgy (host arithmetic only), CT from the CTDI target by a
 * one-rotation run on a CTDI phantom (needs a device).  1 when normalize is 0 or
 * the beam has no target. */
DXMCG_API int dxmcg_beam_calibration(const dxmcg_beam* beam, int correction, const dxmcg_run_options* opts,
    double* factor);

/* ---- world: World<AAVoxelGrid<5, C, 255>> (simulationpipeline.cpp:127-153) ---- */
DXMCG_API int dxmcg_world_create(const int32_t dims[3], const double spacing_cm[3], const dxmcg_material* materials,
    int n_materials, int correction, dxmcg_world** out);
/* AAVoxelGrid::setData(dims, density, material, materials): host arrays of N voxels */
DXMCG_API int dxmcg_world_set_data(dxmcg_world* w, const double* density, const uint8_t* material);
DXMCG_API int dxmcg_world_set_data_f32(dxmcg_world* w, const float* density, const uint8_t* material);
/* World::build(): validate, pack the voxels on the device, tables, majorant */
DXMCG_API int dxmcg_world_build(dxmcg_world* w);
DXMCG_API void dxmcg_world_destroy(dxmcg_world* w);
DXMCG_API int dxmcg_world_clear_tally(dxmcg_world* w);
/* raw tallies: energy imparted (keV), sum of squared deposits, number of events */
DXMCG_API int dxmcg_world_read_tally(dxmcg_world* w, double* energy, double* energy2, uint64_t* count);
/* doseScored(i).dose()/.variance()/.numberOfEvents() for all voxels (simulationpipeline.cpp:174-231), mGy */
DXMCG_API int dxmcg_world_read_dose(dxmcg_world* w, double* dose, double* variance, uint64_t* count);
/* device copy of the FP32 tables (tests): per material photo/incoh/coh/total, majorant */
DXMCG_API int dxmcg_world_tables(dxmcg_world* w, int material, float* xs4, float* majorant);
DXMCG_API int dxmcg_world_packed_density(dxmcg_world* w, float* density, uint8_t* material);

/* ---- transport: Transport::operator()(world, beam, progress, bool) ---------- */
DXMCG_API int dxmcg_transport_run(dxmcg_world* w, const dxmcg_beam* beam, const dxmcg_run_options* opts,
    dxmcg_progress* progress, dxmcg_stats* stats);

/* ---- batches: many (world, beam) jobs in one persistent launch --------------
 * No counterpart in the reference, which runs one beam per Transport call
 * (simulationpipeline.cpp:165).  All jobs draw from one shared history queue, so
 * a batch of small or uneven jobs keeps every SM busy until the last history.
 * Job j runs histories 0..N_j-1 of beams[j] with opts[j].seed and opts[j].stream
 * and deposits into worlds[j]'s tally: the same histories, hence the same tallies
 * up to the summation order, as dxmcg_transport_run(worlds[j], beams + j,
 * opts + j, ...).  A world may appear in several jobs (their doses add).
 * Requirements: every world built and on one device, one tracking mode for all
 * jobs (launch shape from opts[0]), hist_begin = hist_end = 0, one macro_cell
 * per world.  Exposures, spectra and calibrations are fixed at create time; the
 * worlds must outlive the batch and must not run other transports meanwhile.
 * The first dxmcg_batch_run captures a CUDA graph (counter reset + the launch)
 * that every later run replays; each run adds N_j histories to world j's dose
 * normalisation.  stats are summed over all jobs (calibration: job 0's). */
typedef struct dxmcg_batch dxmcg_batch;
DXMCG_API int dxmcg_batch_create(int n_jobs, dxmcg_world* const* worlds, const dxmcg_beam* beams,
    const dxmcg_run_options* opts, dxmcg_batch** out);
/* histories and calibration factor per job (arrays of n_jobs, each may be NULL) */
DXMCG_API int dxmcg_batch_info(const dxmcg_batch* b, int* n_jobs, uint64_t* job_histories, double* job_calibration);
DXMCG_API int dxmcg_batch_run(dxmcg_batch* b, dxmcg_stats* stats);
DXMCG_API void dxmcg_batch_destroy(dxmcg_batch* b);

/* ---- launch-shape autotuner ----------------------------------------------------
 * No counterpart in the reference.  Times the transport kernel on
 * sample_histories (0: 2^24) histories from the middle of the beam for each
 * block size {128, 256} x interact batch {8, 12, 16, 24} x refill batch
 * {4, 8, 16} x Woodcock steps per phase {8, 16} (Woodcock tracking only),
 * depositing into a scratch tally (the world's dose is untouched), and writes the
 * fastest block_size / interact_batch / refill_batch / woodcock_steps into *opts
 * (blocks_per_sm = 0: all resident blocks).  histories_per_second may be NULL. */
DXMCG_API int dxmcg_autotune(dxmcg_world* w, const dxmcg_beam* beam, dxmcg_run_options* opts,
    uint64_t sample_histories, double* histories_per_second);

/* ---- transport that allocates no device memory ------------------------------
 * No counterpart in the reference.  For callers that may not call cudaMalloc or
 * any other device allocator while they run (their GPU memory comes only from
 * their own pool, or they were given a fixed device budget up front): every input
 * and output is a caller-owned device array, and all scratch (queue head,
 * statistics, tables, exposures, spectra, bowtie) lives in one 12 MiB
 * file-scope __device__ array that each GPU loading the library keeps until exit.
 * Limits: at most 16 materials and 4096 exposures (DXMCG_ERR_CAPACITY beyond).
 * CT beams with opts->normalize set and a CTDIvol or CTDIw target are refused
 * (DXMCG_ERR_ARGUMENT): their calibration simulates a CTDI phantom world, which
 * needs device allocations; DX/CBCT (DAP) and pencil (air kerma) calibration work.
 * The first call on a device looks the array up (cudaGetSymbolAddress).  Calls
 * share the array: calls that overlap on the GPU race, so issue them one after
 * another.  The call runs on `cuda_stream` (NULL: the default stream), reads
 * validation results back and synchronises that stream partway, and returns after
 * the stream completes; so no call may be made on a stream that is being captured
 * into a CUDA graph (such a call returns DXMCG_ERR_ARGUMENT before any work).
 * Deposits are added to device_tally (N records, zero it to start afresh);
 * stats->kernel_ms is 0 here and total_ms is the host wall time of the run. */
typedef struct {
    double energy;  /* energy imparted, keV */
    double energy2; /* sum of squared deposits */
    uint64_t count; /* number of deposits */
    uint64_t reserved;
} dxmcg_tally_record;
DXMCG_API int dxmcg_transport_run_noalloc(const int32_t dims[3], const double spacing_cm[3],
    const float* device_density, const uint8_t* device_material, const dxmcg_material* materials, int n_materials,
    int correction, const dxmcg_beam* beam, const dxmcg_run_options* opts, dxmcg_tally_record* device_tally,
    void* cuda_stream, dxmcg_stats* stats);

/* ---- around the transport: segmentation, dose readout, organ dose table ----- */
#define DXMCG_MAX_SEG_MATERIALS 64
/* CTSegmentationPipeline's tables (ctsegmentationpipeline.cpp:59-111): for a tube
 * of kvp with al_mm Al and sn_mm Sn filtration, the spectrum-weighted mean CT
 * number and mass attenuation of each material (ascending CT numbers expected),
 * and of water (1.0 g/cm3) and dry air (0.001205 g/cm3). */
typedef struct {
    int32_t n_materials;
    double hu[DXMCG_MAX_SEG_MATERIALS];
    double separator[DXMCG_MAX_SEG_MATERIALS - 1]; /* (hu[i] + hu[i+1]) / 2 */
    double attenuation[DXMCG_MAX_SEG_MATERIALS];   /* cm2/g */
    double water_attenuation, water_density, air_attenuation, air_density;
} dxmcg_segmentation;
DXMCG_API int dxmcg_ct_segmentation_table(double kvp, double al_mm, double sn_mm, int n_materials,
    const dxmcg_material* materials, const double* densities, dxmcg_segmentation* out);
/* CTSegmentationPipeline::updateImageData's per-voxel pass (:117-160) on the GPU:
 * material = first i with hu < separator[i] (else n_materials - 1), density from the
 * water/air line over the material's attenuation, clamped at 0.  Host arrays of n;
 * the _device form takes device arrays and runs on cuda_stream (NULL: default). */
DXMCG_API int dxmcg_ct_segment(const dxmcg_segmentation* table, const double* hu, uint64_t n, uint8_t* material,
    double* density);
DXMCG_API int dxmcg_ct_segment_device(const dxmcg_segmentation* table, const double* hu, uint64_t n,
    uint8_t* material, double* density, void* cuda_stream);

/* DoseTablePipeline::updateImageData (dosetablepipeline.cpp:55-85): per organ label
 * i < n_organs, voxels, volume (cm3), mass (g) and mean dose = sum(dose x voxel mass)
 * / organ mass, in the dose array's unit.  Labels >= n_organs are ignored; organs
 * without voxels get zeros. */
typedef struct {
    uint64_t n_voxels;
    double volume_cm3;
    double mass_g;
    double dose;
} dxmcg_organ_dose;
DXMCG_API int dxmcg_organ_dose_table(const uint8_t* organ, const double* dose, const double* density, uint64_t n,
    const double spacing_cm[3], int n_organs, dxmcg_organ_dose* out);
DXMCG_API int dxmcg_organ_dose_table_device(const uint8_t* organ, const double* dose, const double* density,
    uint64_t n, const double spacing_cm[3], int n_organs, dxmcg_organ_dose* out, void* cuda_stream);
/* The same table straight from a world's tally (dose in mGy as dxmcg_world_read_dose
 * gives it, mass from the world's stored densities), without a dose array;
 * delete_air_dose: material-0 voxels count with zero dose (simulationpipeline.cpp:180-185). */
DXMCG_API int dxmcg_world_organ_dose(dxmcg_world* w, const uint8_t* organ, int n_organs, int delete_air_dose,
    dxmcg_organ_dose* out);
/* The worker's readout (simulationpipeline.cpp:173-231) on the GPU: dose, variance
 * and event count (as double) with material-0 voxels zeroed when delete_air_dose,
 * and, when the largest dose is below 1 mGy, dose x 1e3 and variance x 1e6 with
 * *micro_gray = 1 (uGy).  Any output may be NULL. */
DXMCG_API int dxmcg_world_read_dose_postprocessed(dxmcg_world* w, int delete_air_dose, double* dose,
    double* variance, double* count, int* micro_gray);

/* ---- dose denoiser ---------------------------------------------------------------
 * No counterpart in the reference.  A 3D convolutional encoder-decoder maps a
 * short run's dose (with the density and material maps) to the converged dose.
 * Levels l = 0..levels-1 at resolution R / 2^l with channels[l] (multiples of 16):
 * two 3x3x3 conv + ReLU per level, 2x2x2 average pooling down, nearest upsampling
 * and concatenation with the level's encoder output up, then a 1x1x1 head.
 * Weights and activations bf16, FP32 accumulation, FP32 master weights and Adam.
 * Tensors are device arrays [B][D][H][W][C] ("channels last"); the input has 16
 * channels: log(1 + dose / scale), density, one-hot of material 0..5, 8 zeros.
 * D, H and W must be multiples of 2^(levels - 1).  Calls take a CUDA stream
 * (NULL: the default stream) and are ordered on it; they return after queuing,
 * except where a host result (loss, parameters) is returned. */
typedef struct dxmcg_denoiser dxmcg_denoiser;
typedef struct {
    int32_t levels;      /* 1..5 */
    int32_t channels[5]; /* per level, multiples of 16; channels[0] 16 or 32 */
    uint64_t seed;       /* He-normal initialisation */
    int32_t conv_path;   /* 3x3x3 convolutions: 0 = default: tcgen05 tensor cores with
                            accumulators in tensor memory, except a launch whose grid would
                            leave SMs idle (fewer output bricks than SMs), which takes mma.sync;
                            1 = tcgen05 for every convolution; 2 = warp-level mma.sync */
} dxmcg_denoiser_config;
DXMCG_API int dxmcg_denoiser_create(const dxmcg_denoiser_config* config, dxmcg_denoiser** out);
DXMCG_API void dxmcg_denoiser_destroy(dxmcg_denoiser* d);
/* Polls of each wait by which one role of the tcgen05 convolution (MMA issue,
 * staging, epilogue) hands work to another before it gives up (0: the default,
 * 2^24; the first poll never blocks).  A convolution that gives up waits for the
 * copies and MMAs it already started, leaves its output unwritten, and the call
 * returns DXMCG_ERR_DEVICE; later calls run normally.  For tests of that path. */
DXMCG_API int dxmcg_denoiser_set_wait_limit(dxmcg_denoiser* d, uint32_t polls);
/* parameters as one FP32 vector: per conv layer (enc0a, enc0b, ..., enc(L-1)b,
 * dec(L-2)a, dec(L-2)b, ..., dec0a, dec0b) weights [Cout][27][Cin] then bias
 * [Cout]; then the head's weights [channels[0]] and bias */
DXMCG_API int dxmcg_denoiser_param_count(const dxmcg_denoiser* d, uint64_t* n);
DXMCG_API int dxmcg_denoiser_get_params(dxmcg_denoiser* d, float* host);
/* sets the parameters and restarts the optimiser (Adam moments and step 0) */
DXMCG_API int dxmcg_denoiser_set_params(dxmcg_denoiser* d, const float* host);
/* gradients of the last dxmcg_denoiser_backward, same layout */
DXMCG_API int dxmcg_denoiser_get_grads(dxmcg_denoiser* d, float* host);
/* pred[B][D][H][W] (FP32, normalised dose) */
DXMCG_API int dxmcg_denoiser_forward(dxmcg_denoiser* d, const void* input, int B, int D, int H, int W, float* pred,
    void* cuda_stream);
/* forward, L1 loss against target[B][D][H][W] and backward; *loss = mean |pred - target| */
DXMCG_API int dxmcg_denoiser_backward(dxmcg_denoiser* d, const void* input, const float* target, int B, int D,
    int H, int W, double* loss, void* cuda_stream);
/* one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) with the last gradients */
DXMCG_API int dxmcg_denoiser_adam(dxmcg_denoiser* d, float lr, void* cuda_stream);
/* the 16 input channels of n voxels from device arrays (dose, density, material) */
DXMCG_API int dxmcg_denoiser_prepare_input(const float* dose, const float* density, const uint8_t* material,
    uint64_t n, double scale, void* input, void* cuda_stream);
/* copy n_patch cubes of edge P into batch tensors: volume v < n_volumes has device
 * input inputs[v] (16 channels) and target targets[v] of dims[3v..3v+2] = (D, H, W);
 * origins[4p..4p+3] = (v, z, y, x); all four arrays in device memory.  Voxels of a
 * patch outside its volume are written as zeros. */
DXMCG_API int dxmcg_denoiser_gather_patches(const void* const* inputs, const float* const* targets,
    const int32_t* dims, int n_volumes, const int32_t* origins, int n_patch, int P, void* input_batch,
    float* target_batch, void* cuda_stream);
/* A world's dose, denoised: input from its tally and voxels (air, material 0, enters
 * with zero dose as the worker's readout deletes it), scale = the mean dose of voxels
 * denser than 0.2 g/cm3 (or `scale` when > 0), dose_out (host, N, mGy as
 * dxmcg_world_read_dose; may be NULL) and *scale_used (may be NULL).  On the tensor-core
 * path the last two convolutions skip output bricks (8 x 16 x 8 voxels) that hold no
 * non-air voxel (the one before: not within one brick of one), and the other layers of
 * levels 0-2 the bricks those do not depend on; the skipped bricks' voxels, all air,
 * get dose 0, and every other voxel the value of the full computation. */
DXMCG_API int dxmcg_world_denoise(dxmcg_world* w, dxmcg_denoiser* d, double scale, double* dose_out,
    double* scale_used);

/* ---- TransportProgress (simulationpipeline.cpp:114-120, :234, :261) ---------- */
DXMCG_API dxmcg_progress* dxmcg_progress_create(void);
DXMCG_API void dxmcg_progress_destroy(dxmcg_progress* p);
DXMCG_API void dxmcg_progress_get(const dxmcg_progress* p, uint64_t* done, uint64_t* total);
DXMCG_API void dxmcg_progress_stop(dxmcg_progress* p);
/* clears a stop request and the counters (a new simulation starts) */
DXMCG_API void dxmcg_progress_reset(dxmcg_progress* p);
DXMCG_API int dxmcg_progress_continue(const dxmcg_progress* p);
DXMCG_API int dxmcg_progress_message(const dxmcg_progress* p, char* buf, int cap);

/* ---- device test hooks: the hot-path pieces run alone on the GPU ------------ */
/* Siddon traversal of n grid-local rays; per ray up to cap segments */
DXMCG_API int dxmcg_siddon_trace(int n_rays, const float* origins, const float* directions, const int32_t dims[3],
    const float spacing[3], int cap, int64_t* voxel, float* length, int32_t* n_segments);
/* first n_draws raw 32-bit draws of the streams of histories h0 .. h0 + n_hist - 1 */
DXMCG_API int dxmcg_history_stream(uint64_t seed, uint32_t stream, uint64_t h0, int n_hist, int n_draws,
    uint32_t* out);
/* samplers driven by injected uniforms (u_stride uniforms per sample) */
DXMCG_API int dxmcg_sample_compton(int n, const double* energies, const dxmcg_material* m, int correction,
    const double* uniforms, int u_stride, double* e_out, double* cos_out, int32_t* used);
DXMCG_API int dxmcg_sample_rayleigh(int n, const double* energies, const dxmcg_material* m, const double* uniforms,
    int u_stride, double* cos_out, int32_t* used);
/* correction level 2 photoelectric absorption: energy of the K fluorescence photon
 * that leaves the atom (0: none) and the z cosine of its isotropic direction */
DXMCG_API int dxmcg_sample_photoelectric(int n, const double* energies, const dxmcg_material* m,
    const double* uniforms, int u_stride, double* e_out, double* dz_out, int32_t* used);
/* tcgen05 self-test (no counterpart in the reference): with A 128 x 16 and B0, B1
 * N x 16 bf16 bit patterns (row-major, N = 16 or 32), d0 = A (B0 + B1)^T and
 * d1 = A B1^T in FP32 [128][N], computed by three tensor-core MMAs into tensor memory */
DXMCG_API int dxmcg_umma_probe(int N, const uint16_t* a, const uint16_t* b0, const uint16_t* b1, float* d0,
    float* d1);
/* source photons of histories [hist_begin, hist_begin + n): E, weight, grid-local pos[3], dir[3] */
DXMCG_API int dxmcg_sample_source(dxmcg_world* w, const dxmcg_beam* beam, const dxmcg_run_options* opts, int n,
    double* out8);

#ifdef __cplusplus
}
#endif
#endif
