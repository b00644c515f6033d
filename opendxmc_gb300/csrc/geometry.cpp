// geometry.cpp -- beam -> exposure expansion (numberOfExposures()/exposure(i),
// beamactorcontainer.cpp:114-121).
//
// DX and pencil beams repeat one pose n_exposures times (the pose is set by
// DXBeam::updatePosition, dxmc_specialization.cpp:78-90; collimation
// half-angles by DXBeam::setCollimation, :46-52).  Rotating beams (CT spiral,
// CT sequential, CBCT, dual-energy spiral) put the source at SDD/2 from the
// isocentre, with c0 along the fan, c1 along the rotation axis and the beam
// direction c0 x c1 pointing at the isocentre -- the same basis
// pointsFromCollimations uses (beamactorcontainer.cpp:44-67).
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/dxmcg.h"
#include "engine.hpp"

namespace dxmcg {
namespace {
    constexpr double kPi = 3.14159265358979323846;

    using V3 = std::array<double, 3>;

    V3 cross(const V3& a, const V3& b)
    {
        return { a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0] };
    }
    double dot(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
    V3 unit(V3 v)
    {
        const double n = std::sqrt(dot(v, v));
        if (n > 0)
            for (auto& x : v)
                x /= n;
        return v;
    }
    // Rodrigues rotation about a unit axis.
    V3 rotate(const V3& v, const V3& k, double angle)
    {
        const V3 kv = cross(k, v);
        const double c = std::cos(angle), s = std::sin(angle), kd = dot(k, v);
        return { v[0] * c + kv[0] * s + k[0] * kd * (1 - c), v[1] * c + kv[1] * s + k[1] * kd * (1 - c),
            v[2] * c + kv[2] * s + k[2] * kd * (1 - c) };
    }

    double profileAt(const double* w, int n, double f)
    {
        if (n <= 0)
            return 1.0;
        if (n == 1)
            return w[0];
        const double x = f * (n - 1);
        if (x <= 0)
            return w[0];
        if (x >= n - 1)
            return w[n - 1];
        const int i = static_cast<int>(x);
        const double t = x - i;
        return w[i] + t * (w[i + 1] - w[i]);
    }

    double aecAt(const dxmcg_beam& b, double z)
    {
        if (b.n_aec <= 0 || !b.aec_weight)
            return 1.0;
        const double z0 = b.aec_start[2], z1 = b.aec_stop[2];
        return profileAt(b.aec_weight, b.n_aec, z1 != z0 ? (z - z0) / (z1 - z0) : 0.0);
    }

    dxmcg_exposure rotatingPose(const V3& iso, const V3& axisIn, double angle, double sid, double halfFan,
        double halfCone)
    {
        const V3 axis = unit(axisIn);
        V3 ref = cross(axis, { 1, 0, 0 });
        if (dot(ref, ref) < 1e-12)
            ref = cross(axis, { 0, 1, 0 });
        ref = unit(ref);
        const V3 s = rotate(ref, axis, angle);
        const V3 dir = { -s[0], -s[1], -s[2] };
        const V3 c0 = cross(axis, dir);
        dxmcg_exposure e {};
        for (int i = 0; i < 3; ++i) {
            e.pos[i] = iso[i] + sid * s[i];
            e.c0[i] = c0[i];
            e.c1[i] = axis[i];
        }
        e.half[0] = halfFan;
        e.half[1] = halfCone;
        e.weight = 1.0;
        e.tube = 0;
        return e;
    }
    // Organ AEC: the tube output is lowered to `low` over the gantry sector
    // [start, stop] (degrees, counter-clockwise, wrapping at 360) and ramps back to 1
    // linearly over `ramp` degrees on both sides.  With compensation the exposures
    // outside the sector and its ramps are raised so that the mean weight is kept.
    void applyOrganAec(const dxmcg_beam& b, const std::vector<double>& angleDeg, std::vector<dxmcg_exposure>& out)
    {
        if (!b.organ_aec || out.empty() || angleDeg.size() != out.size())
            return;
        const auto wrap = [](double a) {
            a = std::fmod(a, 360.0);
            return a < 0 ? a + 360.0 : a;
        };
        const double low = std::min(1.0, std::max(0.0, b.organ_aec_low_weight));
        const double ramp = std::max(0.0, b.organ_aec_ramp_deg);
        const double s0 = wrap(b.organ_aec_start_deg);
        const double span = wrap(b.organ_aec_stop_deg - b.organ_aec_start_deg);
        std::vector<double> f(out.size());
        double lowered = 0.0;
        size_t nOut = 0;
        for (size_t i = 0; i < out.size(); ++i) {
            const double d = wrap(angleDeg[i] - s0);
            if (d <= span) {
                f[i] = low;
            } else {
                const double dist = std::min(d - span, 360.0 - d);
                f[i] = dist < ramp ? low + (1.0 - low) * dist / ramp : 1.0;
            }
            if (f[i] < 1.0)
                lowered += f[i];
            else
                ++nOut;
        }
        if (b.organ_aec_compensate && nOut > 0) {
            const double raise = (static_cast<double>(out.size()) - lowered) / static_cast<double>(nOut);
            for (auto& x : f)
                if (x >= 1.0)
                    x = raise;
        }
        for (size_t i = 0; i < out.size(); ++i)
            out[i].weight *= f[i];
    }
} // namespace

int expandExposures(const dxmcg_beam& b, std::vector<dxmcg_exposure>& out)
{
    out.clear();
    if (b.type == DXMCG_BEAM_DX || b.type == DXMCG_BEAM_PENCIL) {
        const uint64_t n = b.n_exposures > 0 ? b.n_exposures : 1;
        if (n > (1u << 24))
            return DXMCG_ERR_ARGUMENT;
        dxmcg_exposure e {};
        for (int i = 0; i < 3; ++i) {
            e.pos[i] = b.position[i];
            e.c0[i] = b.cosines[0][i];
            e.c1[i] = b.cosines[1][i];
        }
        if (b.type == DXMCG_BEAM_DX) {
            e.half[0] = b.half_angles[0];
            e.half[1] = b.half_angles[1];
        }
        e.weight = 1.0;
        out.assign(n, e);
        return DXMCG_OK;
    }
    if (!(b.sdd_cm > 0) || !(b.step_angle_deg > 0))
        return DXMCG_ERR_ARGUMENT;
    const double sid = 0.5 * b.sdd_cm;
    const double step = b.step_angle_deg * kPi / 180.0;
    const double a0 = b.start_angle_deg * kPi / 180.0;
    const V3 zaxis = { 0, 0, 1 };
    std::vector<double> angles; // gantry angle of every exposure, degrees
    switch (b.type) {
    case DXMCG_BEAM_CT_SPIRAL:
    case DXMCG_BEAM_CT_SPIRAL_DUAL_ENERGY: {
        const double dz = b.stop[2] - b.start[2];
        const double feed = b.collimation_cm * b.pitch;
        if (!(feed > 0))
            return DXMCG_ERR_ARGUMENT;
        const double perRot = 2.0 * kPi / step;
        const long rotations = std::max(1L, static_cast<long>(std::ceil(std::fabs(dz) / feed * perRot - 1e-9)));
        const bool dual = b.type == DXMCG_BEAM_CT_SPIRAL_DUAL_ENERGY;
        const double halfCone = std::atan(0.5 * b.collimation_cm / sid);
        for (long i = 0; i < rotations; ++i) {
            const double angle = a0 + i * step;
            const double z = b.start[2] + (dz >= 0 ? 1.0 : -1.0) * static_cast<double>(i) / perRot * feed;
            const V3 iso = { b.start[0], b.start[1], z };
            for (int t = 0; t < (dual ? 2 : 1); ++t) {
                const double fov = t == 1 ? b.fov_b_cm : b.scan_fov_cm;
                auto e = rotatingPose(iso, zaxis, angle + (t == 1 ? 0.5 * kPi : 0.0), sid, std::atan(0.5 * fov / sid),
                    halfCone);
                e.tube = t;
                const double tubeShare = dual ? (t == 0 ? 2.0 * b.tube_a_weight : 2.0 * (1.0 - b.tube_a_weight)) : 1.0;
                e.weight = aecAt(b, z) * tubeShare;
                out.push_back(e);
                angles.push_back((angle + (t == 1 ? 0.5 * kPi : 0.0)) * 180.0 / kPi);
            }
        }
        break;
    }
    case DXMCG_BEAM_CT_SEQUENTIAL: {
        const long perRot = std::lround(2.0 * kPi / step);
        const int slices = b.n_slices > 0 ? b.n_slices : 1;
        const double halfCone = std::atan(0.5 * b.collimation_cm / sid);
        for (int s = 0; s < slices; ++s) {
            const V3 iso = { b.position[0], b.position[1], b.position[2] + s * b.slice_spacing_cm };
            for (long i = 0; i < perRot; ++i) {
                auto e = rotatingPose(iso, zaxis, a0 + i * step, sid, std::atan(0.5 * b.scan_fov_cm / sid), halfCone);
                e.weight = aecAt(b, iso[2]);
                out.push_back(e);
                angles.push_back((a0 + i * step) * 180.0 / kPi);
            }
        }
        break;
    }
    case DXMCG_BEAM_CBCT: {
        const double a1 = b.stop_angle_deg * kPi / 180.0;
        const long m = std::max(1L, static_cast<long>(std::floor((a1 - a0) / step + 1e-9)) + 1);
        const V3 iso = { b.position[0], b.position[1], b.position[2] };
        const V3 axis = { b.rotation_axis[0], b.rotation_axis[1], b.rotation_axis[2] };
        if (dot(axis, axis) <= 0)
            return DXMCG_ERR_ARGUMENT;
        for (long i = 0; i < m; ++i) {
            out.push_back(rotatingPose(iso, axis, a0 + i * step, sid, b.half_angles[0], b.half_angles[1]));
            angles.push_back((a0 + i * step) * 180.0 / kPi);
        }
        applyOrganAec(b, angles, out); // CBCT exposures carry no z-AEC weight
        return DXMCG_OK;
    }
    default:
        return DXMCG_ERR_ARGUMENT;
    }
    double mean = 0;
    for (const auto& e : out)
        mean += e.weight;
    mean /= static_cast<double>(out.size());
    if (mean > 0)
        for (auto& e : out)
            e.weight /= mean;
    applyOrganAec(b, angles, out);
    return DXMCG_OK;
}

} // namespace dxmcg
