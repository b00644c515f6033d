// dxmc/beams/ctspiralbeam.hpp -- helical CT: start/stop position, pitch, total
// collimation, scan field of view, source-detector distance, start and step angle,
// CTDIvol / CTDI phantom diameter, bowtie, z-AEC and organ AEC
// (beamsettingsmodel.cpp:1139-1340).  The source sits at SDD/2 from the isocentre.
#pragma once

#include "beamtype.hpp"

namespace dxmc {
namespace detail {

    // settings shared by the rotating CT beams
    class CTCommon : public BeamCommon {
    public:
        double sourceDetectorDistance() const { return m_sdd; }
        void setSourceDetectorDistance(double d) { m_sdd = std::abs(d); }
        double collimation() const { return m_coll; }
        void setCollimation(double cm) { m_coll = std::abs(cm); }
        double scanFieldOfView() const { return m_fov; }
        void setScanFieldOfView(double cm) { m_fov = std::abs(cm); }
        double startAngle() const { return m_startDeg * DEG_TO_RAD<double>(); }
        double startAngleDeg() const { return m_startDeg; }
        void setStartAngleDeg(double a) { m_startDeg = a; }
        void setStartAngle(double rad) { m_startDeg = rad * RAD_TO_DEG<double>(); }
        double stepAngleDeg() const { return m_stepDeg; }
        double stepAngle() const { return m_stepDeg * DEG_TO_RAD<double>(); }
        void setStepAngleDeg(double a) { m_stepDeg = std::abs(a) > 0.01 ? std::abs(a) : 0.01; }
        double CTDIdiameter() const { return m_ctdiD; }
        void setCTDIdiameter(double cm) { m_ctdiD = std::abs(cm); }
        const BowtieFilter& bowtieFilter() const { return m_bowtie; }
        void setBowtieFilter(const BowtieFilter& f) { m_bowtie = f; }
        const CTAECFilter& AECFilter() const { return m_aec; }
        void setAECFilter(const CTAECFilter& f) { m_aec = f; }
        CTOrganAECFilter& organAECFilter() { return m_organ; }
        const CTOrganAECFilter& organAECFilter() const { return m_organ; }

    protected:
        void putCommon(dxmcg_beam& b) const
        {
            b.particles_per_exposure = m_ppe;
            b.sdd_cm = m_sdd;
            b.collimation_cm = m_coll;
            b.scan_fov_cm = m_fov;
            b.start_angle_deg = m_startDeg;
            b.step_angle_deg = m_stepDeg;
            b.ctdi_diameter_cm = m_ctdiD;
            putBowtie(b, m_bowtie, m_bowAngle, m_bowWeight);
            putAec(b, m_aec);
            putOrganAec(b, m_organ);
        }

        double m_sdd = 119.0;
        double m_coll = 3.84;
        double m_fov = 50.0;
        double m_startDeg = 0.0;
        double m_stepDeg = 5.0;
        double m_ctdiD = 32.0;
        BowtieFilter m_bowtie;
        CTAECFilter m_aec;
        CTOrganAECFilter m_organ;
    };

} // namespace detail

template <bool ENABLETRACKING = false>
class CTSpiralBeam : public detail::CTCommon {
public:
    CTSpiralBeam(const std::array<double, 3>& start = { 0, 0, 0 }, const std::array<double, 3>& stop = { 0, 0, 0 },
        const std::map<std::size_t, double>& filtrationMaterials = {})
        : m_start(start)
        , m_stop(stop)
    {
        for (const auto& [Z, mm] : filtrationMaterials)
            m_tube.addFiltrationMaterial(Z, mm);
    }

    const std::array<double, 3>& startPosition() const { return m_start; }
    void setStartPosition(const std::array<double, 3>& p) { m_start = p; }
    const std::array<double, 3>& stopPosition() const { return m_stop; }
    void setStopPosition(const std::array<double, 3>& p) { m_stop = p; }
    double pitch() const { return m_pitch; }
    void setPitch(double p) { m_pitch = std::abs(p) > 0.01 ? std::abs(p) : 0.01; }
    double CTDIvol() const { return m_ctdivol; }
    void setCTDIvol(double mgy) { m_ctdivol = std::abs(mgy); }

    Tube& tube() { return m_tube; }
    const Tube& tube() const { return m_tube; }
    void setTubeVoltage(double kvp) { m_tube.setVoltage(kvp); }
    double tubeVoltage() const { return m_tube.voltage(); }
    void setTubeAnodeAngleDeg(double a) { m_tube.setAnodeAngleDeg(a); }
    void addTubeFiltrationMaterial(std::size_t Z, double mm) { m_tube.addFiltrationMaterial(Z, mm); }
    double tubeAlHalfValueLayer() const { return m_tube.mmAlHalfValueLayer(); }
    double tubeMeanSpecterEnergy() const { return m_tube.meanSpecterEnergy(); }

    dxmcg_beam descriptor() const
    {
        dxmcg_beam b {};
        b.type = DXMCG_BEAM_CT_SPIRAL;
        putTube(m_tube, b.kvp, b.n_filters, b.filter_Z, b.filter_mm);
        b.anode_angle_deg = m_tube.anodeAngleDeg();
        putCommon(b);
        for (int i = 0; i < 3; ++i) {
            b.start[i] = m_start[i];
            b.stop[i] = m_stop[i];
        }
        b.pitch = m_pitch;
        b.ctdi_vol_mgy = m_ctdivol;
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
    Tube m_tube { 120.0 };
};

} // namespace dxmc
