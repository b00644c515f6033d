// dxmc/beams/ctspiraldualenergybeam.hpp -- dual-source helical CT: tube A and tube B
// 90 degrees apart, each with its own voltage, filtration, bowtie and field of view,
// output shared by relative mAs (beamsettingsmodel.cpp:1386-1612; exposures
// alternate A, B as drawn at beamactorcontainer.cpp:134-146).
#pragma once

#include "ctspiralbeam.hpp"

namespace dxmc {

template <bool ENABLETRACKING = false>
class CTSpiralDualEnergyBeam : public detail::CTCommon {
public:
    CTSpiralDualEnergyBeam(const std::array<double, 3>& start = { 0, 0, 0 }, const std::array<double, 3>& stop = { 0, 0, 0 },
        const std::map<std::size_t, double>& filtrationMaterialsA = {},
        const std::map<std::size_t, double>& filtrationMaterialsB = {})
        : m_start(start)
        , m_stop(stop)
    {
        for (const auto& [Z, mm] : filtrationMaterialsA)
            m_tubeA.addFiltrationMaterial(Z, mm);
        for (const auto& [Z, mm] : filtrationMaterialsB)
            m_tubeB.addFiltrationMaterial(Z, mm);
    }

    const std::array<double, 3>& startPosition() const { return m_start; }
    void setStartPosition(const std::array<double, 3>& p) { m_start = p; }
    const std::array<double, 3>& stopPosition() const { return m_stop; }
    void setStopPosition(const std::array<double, 3>& p) { m_stop = p; }
    double pitch() const { return m_pitch; }
    void setPitch(double p) { m_pitch = std::abs(p) > 0.01 ? std::abs(p) : 0.01; }
    double CTDIvol() const { return m_ctdivol; }
    void setCTDIvol(double mgy) { m_ctdivol = std::abs(mgy); }
    double scanFieldOfViewA() const { return m_fov; }
    void setScanFieldOfViewA(double cm) { m_fov = std::abs(cm); }
    double scanFieldOfViewB() const { return m_fovB; }
    void setScanFieldOfViewB(double cm) { m_fovB = std::abs(cm); }
    double relativeMasTubeA() const { return m_masA; }
    void setRelativeMasTubeA(double m) { m_masA = std::abs(m); }
    double relativeMasTubeB() const { return m_masB; }
    void setRelativeMasTubeB(double m) { m_masB = std::abs(m); }
    const BowtieFilter& bowtieFilterA() const { return m_bowtie; }
    void setBowtieFilterA(const BowtieFilter& f) { m_bowtie = f; }
    const BowtieFilter& bowtieFilterB() const { return m_bowtieB; }
    void setBowtieFilterB(const BowtieFilter& f) { m_bowtieB = f; }

    Tube& tubeA() { return m_tubeA; }
    const Tube& tubeA() const { return m_tubeA; }
    Tube& tubeB() { return m_tubeB; }
    const Tube& tubeB() const { return m_tubeB; }
    void addTubeAFiltrationMaterial(std::size_t Z, double mm) { m_tubeA.addFiltrationMaterial(Z, mm); }
    void addTubeBFiltrationMaterial(std::size_t Z, double mm) { m_tubeB.addFiltrationMaterial(Z, mm); }
    void setTubeAVoltage(double kvp) { m_tubeA.setVoltage(kvp); }
    void setTubeBVoltage(double kvp) { m_tubeB.setVoltage(kvp); }

    // Tube A's bowtie goes to n_bowtie/bowtie_*, tube B's to n_bowtie_b/bowtie_b_*: the
    // engine weights each tube's photons with its own profile.
    dxmcg_beam descriptor() const
    {
        dxmcg_beam b {};
        b.type = DXMCG_BEAM_CT_SPIRAL_DUAL_ENERGY;
        putTube(m_tubeA, b.kvp, b.n_filters, b.filter_Z, b.filter_mm);
        putTube(m_tubeB, b.kvp_b, b.n_filters_b, b.filter_Z_b, b.filter_mm_b);
        b.anode_angle_deg = m_tubeA.anodeAngleDeg();
        putCommon(b);
        for (int i = 0; i < 3; ++i) {
            b.start[i] = m_start[i];
            b.stop[i] = m_stop[i];
        }
        b.pitch = m_pitch;
        b.ctdi_vol_mgy = m_ctdivol;
        b.fov_b_cm = m_fovB;
        putBowtieInto(m_bowtieB, m_bowAngleB, m_bowWeightB, b.n_bowtie_b, b.bowtie_b_angle, b.bowtie_b_weight);
        const double s = m_masA + m_masB;
        b.tube_a_weight = s > 0 ? m_masA / s : 0.5;
        return b;
    }
    std::uint64_t numberOfExposures() const
    {
        int n = 0;
        const auto b = descriptor();
        dxmcg_beam_exposures(&b, nullptr, 0, &n);
        return static_cast<std::uint64_t>(n);
    }
    std::uint64_t numberOfParticles() const { return numberOfExposures() * m_ppe; }
    Exposure exposure(std::size_t i) const
    {
        const auto ex = expand(descriptor());
        return i < ex.size() ? ex[i] : Exposure {};
    }

private:
    std::array<double, 3> m_start, m_stop;
    double m_pitch = 1.0;
    double m_ctdivol = 1.0;
    double m_fovB = 33.0;
    double m_masA = 1.0, m_masB = 1.0;
    BowtieFilter m_bowtieB;
    mutable std::vector<double> m_bowAngleB, m_bowWeightB; // tube B's profile as the descriptor points at it
    Tube m_tubeA { 140.0 }, m_tubeB { 80.0 };
};

} // namespace dxmc
