// dxmc/beams/cbctbeam.hpp -- cone-beam CT: an arc from start to stop angle about a
// rotation axis through the isocentre, rectangular collimation half-angles, DAP
// (beamsettingsmodel.cpp:718-900).
#pragma once

#include "beamtype.hpp"

namespace dxmc {

template <bool ENABLETRACKING = false>
class CBCTBeam : public detail::BeamCommon {
public:
    CBCTBeam(const std::array<double, 3>& isocenter = { 0, 0, 0 }, const std::array<double, 3>& rotationAxis = { 0, 0, 1 },
        const std::map<std::size_t, double>& filtrationMaterials = {})
        : m_iso(isocenter)
        , m_axis(vectormath::normalized(rotationAxis))
    {
        for (const auto& [Z, mm] : filtrationMaterials)
            m_tube.addFiltrationMaterial(Z, mm);
    }

    const std::array<double, 3>& isocenter() const { return m_iso; }
    void setIsocenter(const std::array<double, 3>& p) { m_iso = p; }
    const std::array<double, 3>& rotationAxis() const { return m_axis; }
    void setRotationAxis(const std::array<double, 3>& a) { m_axis = vectormath::normalized(a); }
    double sourceDetectorDistance() const { return m_sdd; }
    void setSourceDetectorDistance(double d) { m_sdd = std::abs(d); }
    double startAngleDeg() const { return m_startDeg; }
    void setStartAngleDeg(double a) { m_startDeg = a; }
    double stopAngleDeg() const { return m_stopDeg; }
    void setStopAngleDeg(double a) { m_stopDeg = a; }
    double stepAngleDeg() const { return m_stepDeg; }
    void setStepAngleDeg(double a) { m_stepDeg = std::abs(a) > 0.01 ? std::abs(a) : 0.01; }
    const std::array<double, 2>& collimationHalfAngles() const { return m_half; }
    void setCollimationHalfAngles(double x, double y) { m_half = { std::abs(x), std::abs(y) }; }
    void setCollimationHalfAngles(const std::array<double, 2>& a) { setCollimationHalfAngles(a[0], a[1]); }
    std::array<double, 2> collimationHalfAnglesDeg() const
    {
        return { m_half[0] * RAD_TO_DEG<double>(), m_half[1] * RAD_TO_DEG<double>() };
    }
    void setCollimationHalfAnglesDeg(double x, double y)
    {
        setCollimationHalfAngles(x * DEG_TO_RAD<double>(), y * DEG_TO_RAD<double>());
    }
    void setCollimationHalfAnglesDeg(const std::array<double, 2>& a) { setCollimationHalfAnglesDeg(a[0], a[1]); }
    double DAPvalue() const { return m_dap; }
    void setDAPvalue(double dap) { m_dap = std::abs(dap); }
    CTOrganAECFilter& organAECFilter() { return m_organ; }
    const CTOrganAECFilter& organAECFilter() const { return m_organ; }

    Tube& tube() { return m_tube; }
    const Tube& tube() const { return m_tube; }
    void setTubeVoltage(double kvp) { m_tube.setVoltage(kvp); }
    void setTubeAnodeAngleDeg(double a) { m_tube.setAnodeAngleDeg(a); }
    void addTubeFiltrationMaterial(std::size_t Z, double mm) { m_tube.addFiltrationMaterial(Z, mm); }

    dxmcg_beam descriptor() const
    {
        dxmcg_beam b {};
        b.type = DXMCG_BEAM_CBCT;
        putTube(m_tube, b.kvp, b.n_filters, b.filter_Z, b.filter_mm);
        b.anode_angle_deg = m_tube.anodeAngleDeg();
        b.particles_per_exposure = m_ppe;
        for (int i = 0; i < 3; ++i) {
            b.position[i] = m_iso[i];
            b.rotation_axis[i] = m_axis[i];
        }
        b.sdd_cm = m_sdd;
        b.start_angle_deg = m_startDeg;
        b.stop_angle_deg = m_stopDeg;
        b.step_angle_deg = m_stepDeg;
        b.half_angles[0] = m_half[0];
        b.half_angles[1] = m_half[1];
        b.dap_mgycm2 = m_dap;
        putOrganAec(b, m_organ);
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
    std::array<double, 3> m_iso;
    std::array<double, 3> m_axis;
    double m_sdd = 120.0;
    double m_startDeg = -90.0;
    double m_stopDeg = 90.0;
    double m_stepDeg = 1.0;
    std::array<double, 2> m_half { 0.1745, 0.1745 };
    double m_dap = 10.0;
    CTOrganAECFilter m_organ;
    Tube m_tube { 90.0 };
};

} // namespace dxmc
