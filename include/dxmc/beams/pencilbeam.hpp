// dxmc/beams/pencilbeam.hpp -- monoenergetic pencil beam (position, direction,
// energy, air kerma; beamsettingsmodel.cpp:621-716).  With dose normalisation on,
// the engine scales the beam so that its histories, taken as one photon per cm2
// each, carry the set air kerma (dxmcg_beam.air_kerma_mgy).
#pragma once

#include "beamtype.hpp"

namespace dxmc {

template <bool ENABLETRACKING = false>
class PencilBeam : public detail::BeamCommon {
public:
    PencilBeam(const std::array<double, 3>& position = { 0, 0, 0 }, const std::array<double, 3>& direction = { 0, 0, 1 },
        double energy = 60.0)
        : m_pos(position)
        , m_dir(vectormath::normalized(direction))
        , m_energy(energy)
    {
    }

    const std::array<double, 3>& position() const { return m_pos; }
    void setPosition(const std::array<double, 3>& p) { m_pos = p; }
    const std::array<double, 3>& direction() const { return m_dir; }
    void setDirection(const std::array<double, 3>& d) { m_dir = vectormath::normalized(d); }
    double energy() const { return m_energy; }
    void setEnergy(double kev) { m_energy = kev; }
    double airKerma() const { return m_airKerma; }
    void setAirKerma(double mgy) { m_airKerma = std::abs(mgy); }
    std::uint64_t numberOfExposures() const { return m_nexp; }
    void setNumberOfExposures(std::uint64_t n) { m_nexp = n > 0 ? n : 1; }
    std::uint64_t numberOfParticles() const { return m_nexp * m_ppe; }

    dxmcg_beam descriptor() const
    {
        dxmcg_beam b {};
        b.type = DXMCG_BEAM_PENCIL;
        b.energy_kev = m_energy;
        b.particles_per_exposure = m_ppe;
        b.n_exposures = m_nexp;
        b.air_kerma_mgy = m_airKerma;
        // any orthonormal pair with c0 x c1 = direction
        std::array<double, 3> ref = std::abs(m_dir[2]) < 0.9 ? std::array<double, 3> { 0, 0, 1 }
                                                              : std::array<double, 3> { 1, 0, 0 };
        const auto c0 = vectormath::normalized(vectormath::cross(ref, m_dir));
        const auto c1 = vectormath::cross(m_dir, c0);
        for (int i = 0; i < 3; ++i) {
            b.position[i] = m_pos[i];
            b.cosines[0][i] = c0[i];
            b.cosines[1][i] = c1[i];
        }
        return b;
    }
    Exposure exposure(std::size_t i) const
    {
        const auto ex = expand(descriptor());
        return i < ex.size() ? ex[i] : Exposure {};
    }

private:
    std::array<double, 3> m_pos;
    std::array<double, 3> m_dir;
    double m_energy;
    double m_airKerma = 1.0;
    std::uint64_t m_nexp = 10;
};

} // namespace dxmc
