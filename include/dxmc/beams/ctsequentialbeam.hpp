// dxmc/beams/ctsequentialbeam.hpp -- axial CT: full rotations at numberOfSlices()
// positions sliceSpacing() apart along the scan normal (beamsettingsmodel.cpp:902-1137).
// The engine steps the slices along +z; the scan normal is kept for source compatibility.
#pragma once

#include "ctspiralbeam.hpp"

namespace dxmc {

template <bool ENABLETRACKING = false>
class CTSequentialBeam : public detail::CTCommon {
public:
    CTSequentialBeam(const std::array<double, 3>& position = { 0, 0, 0 },
        const std::array<double, 3>& scanNormal = { 0, 0, 1 }, const std::map<std::size_t, double>& filtrationMaterials = {})
        : m_position(position)
        , m_normal(vectormath::normalized(scanNormal))
    {
        for (const auto& [Z, mm] : filtrationMaterials)
            m_tube.addFiltrationMaterial(Z, mm);
    }

    const std::array<double, 3>& position() const { return m_position; }
    void setPosition(const std::array<double, 3>& p) { m_position = p; }
    const std::array<double, 3>& scanNormal() const { return m_normal; }
    void setScanNormal(const std::array<double, 3>& n) { m_normal = vectormath::normalized(n); }
    std::uint64_t numberOfSlices() const { return m_slices; }
    void setNumberOfSlices(std::uint64_t n) { m_slices = n > 0 ? n : 1; }
    double sliceSpacing() const { return m_spacing; }
    void setSliceSpacing(double cm) { m_spacing = std::abs(cm); }
    double CTDIw() const { return m_ctdiw; }
    void setCTDIw(double mgy) { m_ctdiw = std::abs(mgy); }

    Tube& tube() { return m_tube; }
    const Tube& tube() const { return m_tube; }
    void setTubeVoltage(double kvp) { m_tube.setVoltage(kvp); }
    double tubeVoltage() const { return m_tube.voltage(); }
    void setTubeAnodeAngleDeg(double a) { m_tube.setAnodeAngleDeg(a); }
    void addTubeFiltrationMaterial(std::size_t Z, double mm) { m_tube.addFiltrationMaterial(Z, mm); }

    dxmcg_beam descriptor() const
    {
        dxmcg_beam b {};
        b.type = DXMCG_BEAM_CT_SEQUENTIAL;
        putTube(m_tube, b.kvp, b.n_filters, b.filter_Z, b.filter_mm);
        b.anode_angle_deg = m_tube.anodeAngleDeg();
        putCommon(b);
        for (int i = 0; i < 3; ++i)
            b.position[i] = m_position[i];
        b.n_slices = static_cast<int32_t>(m_slices);
        b.slice_spacing_cm = m_spacing;
        b.ctdi_w_mgy = m_ctdiw;
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
    std::array<double, 3> m_position;
    std::array<double, 3> m_normal;
    std::uint64_t m_slices = 1;
    double m_spacing = 1.0;
    double m_ctdiw = 1.0;
    Tube m_tube { 120.0 };
};

} // namespace dxmc
