// physics.hpp -- host-side (FP64) photon interaction model, material tables and
// X-ray tube spectrum.  These feed the device tables built at World::build()
// (simulationpipeline.cpp:146-153) and the Tube API (ctsegmentationpipeline.cpp:66-71).
//
// The model is project-authored and parametric (DXMClib's Livermore/EPDL data are
// not available to this project):
//  * Compton: Klein-Nishina, times the incoherent scattering function S(x, Z) when
//    the low-energy correction level is >= 1;
//  * Rayleigh: Thomson times the atomic form factor F(x, Z)^2;
//  * F = Z / (1 + x^2/a_Z)^2 and S = Z (1 - (F/Z)^2): one hydrogen-like orbital with the
//    Thomas-Fermi radius scaling, a_Z = (Z^(1/3) / (2 pi a0))^2, x = sin(theta/2)/lambda [1/A];
//  * photoelectric: C Z^4 / E^3 with K/L edges at Moseley energies and jump ratios;
//  * tube: Kramers' thick-target law on 1 keV bins plus tungsten K lines with
//    Green-Cosslett yield scaling, exponential filtration.
#pragma once

#include <array>
#include <cstdint>
#include <vector>

#include "../../include/dxmcg.h"

namespace dxmcg {

constexpr int kNE = DXMCG_NE;
constexpr double kEmin = 1.0;
constexpr double kDE = 0.5;
constexpr double kEcut = 1.0;

namespace phys {
    double atomicMass(int Z);
    double elementDensity(int Z);
    double kleinNishinaTotal(double E);       // barn per electron
    double photoelectric(double E, int Z);    // barn per atom
    double incoherent(double E, int Z, int correction);
    double coherent(double E, int Z);
    double knEnergyTransferFraction(double E);
    double formFactorScale(int Z);            // a_Z in 1/A^2
}

// Composition -> mass attenuation (cm^2/g) at arbitrary energies.
struct Attenuation {
    double photo = 0, incoherent = 0, coherent = 0;
    double sum() const { return photo + incoherent + coherent; }
};
bool validComposition(const dxmcg_material& m);
Attenuation attenuation(const dxmcg_material& m, int correction, double E);

// Per-element data the device samplers use (n_i = w_i / A_i).
struct SamplingElements {
    int n = 0;
    std::array<double, DXMCG_MAX_ELEMENTS> nZ {}, nZ2 {}, a {};
    double Zsum = 0;
};
SamplingElements samplingElements(const dxmcg_material& m);

struct Spectrum {
    std::vector<double> energy;
    std::vector<double> weight; // normalised to 1
};
Spectrum tubeSpectrum(double kvp, double anode_angle_deg, int n_filters, const int32_t* Z, const double* mm);
double tubeMeanEnergy(const Spectrum& s);
double tubeAlHalfValueLayer(const Spectrum& s);
double airEnergyAbsorption(double E); // cm^2/g, mu_tr of dry air (for DAP normalisation)

// Walker alias table with 23-bit integer acceptance thresholds.
struct AliasTable {
    std::vector<float> energy;
    std::vector<uint32_t> threshold;
    std::vector<int32_t> alias;
};
AliasTable buildAlias(const Spectrum& s);

} // namespace dxmcg
