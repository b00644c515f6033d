// dxmc/beams/beamtype.hpp -- what every beam of the dxmc:: layer shares: the
// exposure type (exposure(i).position()/directionCosines()/collimationHalfAngles(),
// beamactorcontainer.cpp:114-121, :134-146) and the conversion of a beam's settings
// into the engine's dxmcg_beam descriptor.
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <vector>

#include "../../dxmcg.h"
#include "../floating.hpp"
#include "../vectormath.hpp"
#include "filters/bowtiefilter.hpp"
#include "filters/ctaecfilter.hpp"
#include "tube/tube.hpp"

namespace dxmc {

class Exposure {
public:
    Exposure() = default;
    Exposure(const dxmcg_exposure& e, std::uint64_t histories)
        : m_e(e)
        , m_histories(histories)
    {
    }
    std::array<double, 3> position() const { return { m_e.pos[0], m_e.pos[1], m_e.pos[2] }; }
    std::array<std::array<double, 3>, 2> directionCosines() const
    {
        return { { { m_e.c0[0], m_e.c0[1], m_e.c0[2] }, { m_e.c1[0], m_e.c1[1], m_e.c1[2] } } };
    }
    std::array<double, 3> direction() const { return vectormath::cross(directionCosines()[0], directionCosines()[1]); }
    std::array<double, 2> collimationHalfAngles() const { return { m_e.half[0], m_e.half[1] }; }
    double beamIntensityWeight() const { return m_e.weight; }
    std::uint64_t numberOfHistories() const { return m_histories; }

private:
    dxmcg_exposure m_e {};
    std::uint64_t m_histories = 0;
};

namespace detail {

    // Settings every beam keeps, and the descriptor filling they share.
    class BeamCommon {
    public:
        std::uint64_t numberOfParticlesPerExposure() const { return m_ppe; }
        void setNumberOfParticlesPerExposure(std::uint64_t n) { m_ppe = n > 0 ? n : 1; }

    protected:
        static void putTube(const Tube& t, double& kvp, int32_t& n, int32_t* Z, double* mm)
        {
            kvp = t.voltage();
            n = t.filters(Z, mm);
        }
        // the profile's points into (ang, w), which must outlive the descriptor, and
        // the descriptor's (n, angles, weights) fields pointing at them
        static void putBowtieInto(const BowtieFilter& f, std::vector<double>& ang, std::vector<double>& w, int32_t& n,
            const double*& angles, const double*& weights)
        {
            ang.clear();
            w.clear();
            for (const auto& [a, v] : f.data()) {
                ang.push_back(a);
                w.push_back(v);
            }
            n = static_cast<int32_t>(ang.size());
            angles = ang.empty() ? nullptr : ang.data();
            weights = w.empty() ? nullptr : w.data();
        }
        void putBowtie(dxmcg_beam& b, const BowtieFilter& f, std::vector<double>& ang, std::vector<double>& w) const
        {
            putBowtieInto(f, ang, w, b.n_bowtie, b.bowtie_angle, b.bowtie_weight);
        }
        static void putAec(dxmcg_beam& b, const CTAECFilter& f)
        {
            if (f.isEmpty())
                return;
            b.n_aec = static_cast<int32_t>(f.weights().size());
            for (int i = 0; i < 3; ++i) {
                b.aec_start[i] = f.startPosition()[i];
                b.aec_stop[i] = f.stopPosition()[i];
            }
            b.aec_weight = f.weights().data();
        }
        static void putOrganAec(dxmcg_beam& b, const CTOrganAECFilter& f)
        {
            b.organ_aec = f.useFilter() ? 1 : 0;
            b.organ_aec_start_deg = f.startAngleDeg();
            b.organ_aec_stop_deg = f.stopAngleDeg();
            b.organ_aec_ramp_deg = f.rampAngleDeg();
            b.organ_aec_low_weight = f.lowWeightFactor();
            b.organ_aec_compensate = f.compensateOutside() ? 1 : 0;
        }
        static std::vector<Exposure> expand(const dxmcg_beam& b)
        {
            int n = 0;
            std::vector<Exposure> out;
            if (dxmcg_beam_exposures(&b, nullptr, 0, &n) != DXMCG_OK || n <= 0)
                return out;
            std::vector<dxmcg_exposure> ex(static_cast<std::size_t>(n));
            dxmcg_beam_exposures(&b, ex.data(), n, &n);
            for (const auto& e : ex)
                out.emplace_back(e, b.particles_per_exposure);
            return out;
        }

        std::uint64_t m_ppe = 1000000;
        // storage the descriptor points into
        mutable std::vector<double> m_bowAngle, m_bowWeight;
    };

} // namespace detail
} // namespace dxmc
