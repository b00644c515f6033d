// dxmc/beams/dxbeam.hpp -- planar (DX) beam: one source pose repeated over
// numberOfExposures() exposures.  Constructor and setters as OpenDXMC's DXBeam wrapper
// uses them (dxmc_specialization.cpp:21-90) and as the beam settings edit them
// (beamsettingsmodel.cpp:459-620).
#pragma once

#include "beamtype.hpp"

namespace dxmc {

template <bool ENABLETRACKING = false>
class DXBeam : public detail::BeamCommon {
public:
    DXBeam(const std::array<double, 3>& pos = { 0, 0, 0 },
        const std::array<std::array<double, 3>, 2>& dircosines = { { { 1, 0, 0 }, { 0, 1, 0 } } },
        const std::map<std::size_t, double>& filtrationMaterials = {})
        : m_pos(pos)
        , m_dircosines(dircosines)
    {
        for (const auto& [Z, mm] : filtrationMaterials)
            m_tube.addFiltrationMaterial(Z, mm);
    }

    const std::array<double, 3>& position() const { return m_pos; }
    void setPosition(const std::array<double, 3>& p) { m_pos = p; }
    const std::array<std::array<double, 3>, 2>& directionCosines() const { return m_dircosines; }
    void setDirectionCosines(const std::array<std::array<double, 3>, 2>& c)
    {
        m_dircosines = { vectormath::normalized(c[0]), vectormath::normalized(c[1]) };
    }
    std::array<double, 3> direction() const { return vectormath::cross(m_dircosines[0], m_dircosines[1]); }

    const std::array<double, 2>& collimationHalfAngles() const { return m_half; }
    void setCollimationHalfAngles(const std::array<double, 2>& a) { m_half = { std::abs(a[0]), std::abs(a[1]) }; }
    void setCollimationHalfAngles(double x, double y) { setCollimationHalfAngles(std::array<double, 2> { x, y }); }
    std::array<double, 2> collimationHalfAnglesDeg() const
    {
        return { m_half[0] * RAD_TO_DEG<double>(), m_half[1] * RAD_TO_DEG<double>() };
    }
    void setCollimationHalfAnglesDeg(const std::array<double, 2>& a)
    {
        setCollimationHalfAngles(a[0] * DEG_TO_RAD<double>(), a[1] * DEG_TO_RAD<double>());
    }
    void setCollimationHalfAnglesDeg(double x, double y) { setCollimationHalfAnglesDeg(std::array<double, 2> { x, y }); }

    std::uint64_t numberOfExposures() const { return m_nexp; }
    void setNumberOfExposures(std::uint64_t n) { m_nexp = n > 0 ? n : 1; }
    std::uint64_t numberOfParticles() const { return m_nexp * m_ppe; }

    Tube& tube() { return m_tube; }
    const Tube& tube() const { return m_tube; }
    void setTubeVoltage(double kvp) { m_tube.setVoltage(kvp); }
    double tubeVoltage() const { return m_tube.voltage(); }
    void setTubeAnodeAngleDeg(double a) { m_tube.setAnodeAngleDeg(a); }
    double tubeAnodeAngleDeg() const { return m_tube.anodeAngleDeg(); }
    void addTubeFiltrationMaterial(std::size_t Z, double mm) { m_tube.addFiltrationMaterial(Z, mm); }
    double tubeAlHalfValueLayer() const { return m_tube.mmAlHalfValueLayer(); }
    double tubeMeanSpecterEnergy() const { return m_tube.meanSpecterEnergy(); }

    double DAPvalue() const { return m_dap; }
    void setDAPvalue(double dap) { m_dap = std::abs(dap); }

    dxmcg_beam descriptor() const
    {
        dxmcg_beam b {};
        b.type = DXMCG_BEAM_DX;
        putTube(m_tube, b.kvp, b.n_filters, b.filter_Z, b.filter_mm);
        b.anode_angle_deg = m_tube.anodeAngleDeg();
        b.particles_per_exposure = m_ppe;
        b.n_exposures = m_nexp;
        for (int i = 0; i < 3; ++i) {
            b.position[i] = m_pos[i];
            b.cosines[0][i] = m_dircosines[0][i];
            b.cosines[1][i] = m_dircosines[1][i];
        }
        b.half_angles[0] = m_half[0];
        b.half_angles[1] = m_half[1];
        b.dap_mgycm2 = m_dap;
        return b;
    }
    Exposure exposure(std::size_t i) const
    {
        const auto ex = expand(descriptor());
        return i < ex.size() ? ex[i] : Exposure {};
    }

private:
    std::array<double, 3> m_pos;
    std::array<std::array<double, 3>, 2> m_dircosines;
    std::array<double, 2> m_half { 0.0, 0.0 };
    std::uint64_t m_nexp = 10;
    double m_dap = 10.0;
    Tube m_tube { 120.0 };
};

} // namespace dxmc
