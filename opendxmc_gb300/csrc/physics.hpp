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
//    Green-Cosslett yield scaling, exponential filtration;
//  * correction level 2 (impulse approximation, simulationwidget.cpp:68-73): each
//    element has three Compton shells (K: min(Z, 2) electrons bound by the Moseley K
//    edge; L: up to 8 electrons bound by Ryd max(Z - 7.4, Z/2)^2 / 4; the rest bound by
//    Ryd (Z/3)^2 / 9), each with the hydrogen-like 1s Compton profile
//    J(p) ~ (1 + (p/p_s)^2)^-3 whose momentum scale p_s = sqrt(U_s / Ryd) atomic units
//    follows from its binding energy U_s; a photoelectric absorption above the K edge
//    leaves a K vacancy with probability 1 - 1/J_K, which emits a K-alpha photon of
//    0.75 Ryd (Z - 1)^2 with the yield omega_K(Z) of Bambynek et al. (Rev. Mod. Phys.
//    44, 716, 1972): omega = X^4 / (1 + X^4), X = 0.015 + 0.0327 Z - 0.64e-6 Z^3.
//
// Physics tables.  A table file replaces the model's numbers element by element
// (elements it does not list keep the model) and may add unfiltered tube spectra.
// It is plain text, whitespace-separated, '#' starts a comment:
//
//   dxmcg-physics 1
//   energies <n> <E_1> ... <E_n>          keV, ascending; a repeated energy marks an
//                                          absorption edge (below, then above it)
//   element <Z> <A>                        atomic number, atomic mass (g/mol)
//     photo <n values>                     photoelectric, barn/atom, at the energies
//     incoherent <n values>                Compton with binding (correction >= 1)
//     incoherent_free <n values>           Compton of free electrons (correction 0;
//                                          optional: Z x Klein-Nishina when absent)
//     coherent <n values>                  Rayleigh
//     formfactor <a_Z>                     1/A^2 scale of F and S in the samplers
//     edges <K keV> <L keV>
//     fluorescence <K-alpha keV> <omega_K>
//     shells <m> (<electrons> <binding keV> <momentum m_e c>) x m    (m <= 3)
//   end
//   tube <kVp> <anode angle deg> <m> (<E keV> <photons>) x m
//
// Cross sections between the listed energies are interpolated linearly in log E and
// log sigma (linearly where a value is 0), and held at the end values outside them;
// at a listed energy the listed value is returned exactly.  A tube entry replaces
// the unfiltered spectrum of that exact (kVp, anode angle); filtration is applied as
// usual.  Loaded tables take effect for worlds built and spectra made afterwards.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dxmcg.h"

namespace dxmcg {

constexpr int kNE = DXMCG_NE;
constexpr double kEmin = 1.0;
constexpr double kDE = 0.5;
constexpr double kEcut = 1.0;

namespace phys {
    constexpr double kJumpRatioK = 7.0; // photoelectric jump ratios at the K and L edges
    constexpr double kJumpRatioL = 3.0;
    double atomicMass(int Z);
    double elementDensity(int Z);
    double kleinNishinaTotal(double E);       // barn per electron
    double photoelectric(double E, int Z);    // barn per atom
    double incoherent(double E, int Z, int correction);
    double coherent(double E, int Z);
    double knEnergyTransferFraction(double E);
    double formFactorScale(int Z);            // a_Z in 1/A^2
    double kEdge(int Z);                      // keV
    double lEdge(int Z);                      // keV, 0 for Z <= 7
    double kAlphaEnergy(int Z);               // keV
    double fluorescenceYieldK(int Z);
    // correction level 2 Compton shells: electrons, binding energy (keV) and the
    // momentum scale of the profile in units of m_e c
    struct Shells {
        int n = 0;
        double electrons[3] {}, binding[3] {}, momentum[3] {};
    };
    Shells comptonShells(int Z);
}

// Physics tables (format above): load replaces the current table (reset: the model
// alone); write dumps the current numbers of the given elements on the attenuation
// table grid (1.0 + 0.5 i keV, i < DXMCG_NE).  Each load or reset increments the
// generation, which the caches keyed on element data compare against.
int loadPhysicsTable(const std::string& path, std::string& err);
void resetPhysicsTable();
int writePhysicsTable(const std::string& path, int n, const int32_t* Z, std::string& err);
uint64_t physicsGeneration();

// Composition -> mass attenuation (cm^2/g) at arbitrary energies.
struct Attenuation {
    double photo = 0, incoherent = 0, coherent = 0;
    double sum() const { return photo + incoherent + coherent; }
};
bool validComposition(const dxmcg_material& m);
Attenuation attenuation(const dxmcg_material& m, int correction, double E);

// Per-element data the device samplers use (n_i = w_i / A_i).  Correction level 2
// adds per element n_i Z^4 (the photoelectric share up to the common C / E^3), the K
// and L edges, the K-alpha energy and the K fluorescence yield, and the material's
// Compton shells (electrons n_i x occupancy, binding, momentum scale).
constexpr int kMaxShells = 3 * DXMCG_MAX_ELEMENTS;
struct SamplingElements {
    int n = 0;
    std::array<double, DXMCG_MAX_ELEMENTS> nZ {}, nZ2 {}, a {};
    std::array<double, DXMCG_MAX_ELEMENTS> nZ4 {}, eK {}, eL {}, kAlpha {}, omegaK {};
    double Zsum = 0;
    int nShell = 0;
    std::array<double, kMaxShells> shellElectrons {}, shellBinding {}, shellMomentum {};
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
