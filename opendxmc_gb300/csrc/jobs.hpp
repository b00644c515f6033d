// jobs.hpp -- host-side preparation of what one transport launch needs, shared by
// the world-based entry points (capi.cpp) and the allocation-free entry point
// (noalloc.cu): per-material FP32 tables and majorant, exposures in grid-local
// coordinates, spectrum alias tables, the bowtie profile.
#pragma once

#include <string>
#include <vector>

#include "engine.hpp"
#include "physics.hpp"

namespace dxmcg {

struct HostJob {
    std::vector<DevExposure> exposures;
    DevSpectrum spec[2];
    bool hasBowtie = false;
    DevBowtie bowtie {};
    uint64_t nHist = 0;
};

// Beam -> exposures, spectra, bowtie for a grid of dims x spacing centred on the
// origin.  Returns DXMCG_OK or an error code with `err` set.
int buildHostJob(const dxmcg_beam& b, const int32_t dims[3], const double spacing[3], HostJob& out, std::string& err);

// Grid, stream and beam fields of a DevJob (device pointers are set by the caller).
void fillJobFields(DevJob& J, const dxmcg_beam& b, const dxmcg_run_options& o, const int32_t dims[3],
    const double spacing[3], int correction, int n_mats, int n_exp);

// Mass attenuation of one material on the table grid (FP64), from per-element
// tables cached for the life of the process.
void materialTables(const dxmcg_material& m, int correction, double* photo, double* incoh, double* coh);

// FP32 device tables for M materials and the majorant (rho_max[m] * total, times a
// small safety factor, maximised over m) on the table grid.
// majorant of material 0 alone: rho0 x its total attenuation, with the same safety
// factor and floor as the grid's majorant
void buildBackgroundMajorant(const float* tot0, double rho0, float* out);
// Compton and Rayleigh angle quantiles out[m][i][j] (kCTabK per row; see kCTabK),
// kept per (composition, correction) for the life of the physics tables
void buildComptonAngleTables(const dxmcg_material* mats, int M, int correction, float* out);
void buildRayleighAngleTables(const dxmcg_material* mats, int M, float* out);
// two-region Woodcock: the box {lo x, y, z, hi x, y, z} of the voxels whose material is
// neither 0 nor transparent (hi x = -1: none) is worth a second region when it leaves
// part of the grid out; setTwoRegion fills J's box fields and material 0's majorant
bool twoRegionBox(const int box[6], const int32_t dims[3]);
// the box's share of the grid's voxels (0 without a box)
double boxFraction(const int box[6], const int32_t dims[3]);
// whether Woodcock runs with two regions: two_region 1 on, -1 off, 0 on when the box
// holds less than half the grid.  Measured: on at box fractions 0.44 (256x256x200
// torso, +13 %) and 0.36 (512x512x400 torso, +23 %); off at 0.53-0.62 (the batch
// workload's ellipsoids, -12 %) and 0.94 (the DX cylinder, -11 %).
bool twoRegionFor(const dxmcg_run_options& o, double boxFrac);
void setTwoRegion(DevJob& J, const int box[6], const double spacing[3], const float* majOut);
void buildDeviceTables(const dxmcg_material* mats, int M, int correction, const double* rhoMax, float* tot,
    float4* xs, float* maj, DevMaterial* dm);

DevMaterial toDevMaterial(const dxmcg_material& m);


} // namespace dxmcg
