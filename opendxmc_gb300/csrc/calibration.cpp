// calibration.cpp -- dose calibration of a beam (the trailing `true` of
// transport(world, beam, progress, true), simulationpipeline.cpp:165), applied when
// dxmcg_run_options.normalize is set: every history weight of the run is multiplied
// by one factor F so that the tallies refer to the beam's calibration quantity.
//
//  * DX, CBCT (setDAPvalue, beamsettingsmodel.cpp:576): the dose-area product of a
//    point source is the same at every distance, E (mu_tr/rho)_air per photon, so
//    F = DAP / (N * sum_k p_k E_k (mu_tr/rho)_air(E_k)) over the N histories of the beam.
//  * CT spiral / sequential / dual energy (setCTDIvol, setCTDIw, setCTDIdiameter,
//    :1054, :1278-1293): one rotation of the same tube, bowtie and geometry is
//    simulated on a generated PMMA cylinder (diameter ctdi_diameter_cm, default 32 cm,
//    15 cm long); dose to PMMA is scored in five 1.31 cm diameter, 10 cm long chamber
//    volumes (centre and 1 cm below the surface at 0/90/180/270 degrees);
//    CTDI100 = D_avg * 10 cm / collimation, CTDIw = CTDI100_c / 3 + 2 / 3 mean(CTDI100_p),
//    CTDIvol = CTDIw / pitch (spiral) or CTDIw * collimation / slice spacing
//    (sequential).  F = CTDIw_target / (CTDIw per history-per-rotation * histories
//    per rotation of the beam).
//  * pencil beams (setAirKerma, beamsettingsmodel.cpp:675): the air kerma of a fluence
//    of one photon per cm2 is E (mu_tr/rho)_air, so with the target air kerma K of the
//    beam's N histories taken as N photons per cm2, F = K / (N E (mu_tr/rho)_air(E)).
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/dxmcg.h"
#include "engine.hpp"
#include "physics.hpp"

namespace dxmcg {
namespace {
    constexpr double kKeVToMilliGrayGram = 1.602176634e-10;
    constexpr double kPi = 3.14159265358979323846;
    constexpr uint64_t kCtdiHistories = 8ull << 20;

    dxmcg_material pmma()
    {
        // C5H8O2 by mass: H 8.054 %, C 59.985 %, O 31.961 %
        dxmcg_material m {};
        m.n = 3;
        m.Z[0] = 1;
        m.w[0] = 8.054;
        m.Z[1] = 6;
        m.w[1] = 59.985;
        m.Z[2] = 8;
        m.w[2] = 31.961;
        return m;
    }

    dxmcg_material dryAir()
    {
        dxmcg_material m {};
        m.n = 3;
        m.Z[0] = 7;
        m.w[0] = 75.5;
        m.Z[1] = 8;
        m.w[1] = 23.2;
        m.Z[2] = 18;
        m.w[2] = 1.3;
        return m;
    }

    bool isCt(int type)
    {
        return type == DXMCG_BEAM_CT_SPIRAL || type == DXMCG_BEAM_CT_SEQUENTIAL
            || type == DXMCG_BEAM_CT_SPIRAL_DUAL_ENERGY;
    }

    long viewsPerRotation(const dxmcg_beam& b) { return std::lround(360.0 / b.step_angle_deg); }

    struct WorldGuard {
        dxmcg_world* w = nullptr;
        ~WorldGuard() { dxmcg_world_destroy(w); }
    };

    // CTDIw (mGy) per history of a one-rotation run of the beam's tube and geometry.
    int ctdiwPerHistory(const dxmcg_beam& b, int correction, uint64_t seed, double& out, std::string& err)
    {
        const double D = b.ctdi_diameter_cm > 0 ? b.ctdi_diameter_cm : 32.0;
        const double R = 0.5 * D;
        const double sxy = 0.1, sz = 0.5;
        const int nxy = 2 * static_cast<int>(std::ceil((R + 1.0) / sxy));
        const int nz = 30; // 15 cm
        const size_t N = static_cast<size_t>(nxy) * nxy * nz;
        std::vector<double> dens(N);
        std::vector<uint8_t> mat(N);
        std::vector<int8_t> region(N, -1);
        const double holeR = 0.5 * 1.31;
        const double cx[5] = { 0.0, 0.0, R - 1.0, 0.0, -(R - 1.0) };
        const double cy[5] = { 0.0, R - 1.0, 0.0, -(R - 1.0), 0.0 };
        for (int k = 0; k < nz; ++k) {
            const double z = (k + 0.5) * sz - 0.5 * nz * sz;
            for (int j = 0; j < nxy; ++j) {
                const double y = (j + 0.5) * sxy - 0.5 * nxy * sxy;
                for (int i = 0; i < nxy; ++i) {
                    const double x = (i + 0.5) * sxy - 0.5 * nxy * sxy;
                    const size_t v = i + static_cast<size_t>(nxy) * (j + static_cast<size_t>(nxy) * k);
                    const bool inPmma = x * x + y * y <= R * R;
                    mat[v] = inPmma ? 1 : 0;
                    dens[v] = inPmma ? 1.19 : 0.0012;
                    if (inPmma && std::fabs(z) <= 5.0)
                        for (int r = 0; r < 5; ++r)
                            if ((x - cx[r]) * (x - cx[r]) + (y - cy[r]) * (y - cy[r]) <= holeR * holeR)
                                region[v] = static_cast<int8_t>(r);
                }
            }
        }
        const int32_t dims[3] = { nxy, nxy, nz };
        const double spacing[3] = { sxy, sxy, sz };
        const dxmcg_material mats[2] = { dryAir(), pmma() };
        WorldGuard g;
        int rc = dxmcg_world_create(dims, spacing, mats, 2, correction, &g.w);
        if (rc == DXMCG_OK)
            rc = dxmcg_world_set_data(g.w, dens.data(), mat.data());
        if (rc == DXMCG_OK)
            rc = dxmcg_world_build(g.w);
        if (rc != DXMCG_OK) {
            err = std::string("CTDI phantom: ") + dxmcg_last_error();
            return rc;
        }
        // one rotation at the phantom centre, no z- or organ-AEC
        dxmcg_beam c = b;
        c.n_aec = 0;
        c.aec_weight = nullptr;
        c.organ_aec = 0;
        const bool dual = b.type == DXMCG_BEAM_CT_SPIRAL_DUAL_ENERGY;
        if (dual) {
            const double feed = b.collimation_cm * b.pitch;
            c.start[0] = c.start[1] = c.stop[0] = c.stop[1] = 0.0;
            c.start[2] = -0.5 * feed;
            c.stop[2] = 0.5 * feed;
        } else {
            c.type = DXMCG_BEAM_CT_SEQUENTIAL;
            c.position[0] = c.position[1] = c.position[2] = 0.0;
            c.n_slices = 1;
        }
        const uint64_t views = static_cast<uint64_t>(viewsPerRotation(b)) * (dual ? 2 : 1);
        c.particles_per_exposure = std::max<uint64_t>(1, kCtdiHistories / views);
        dxmcg_run_options o {};
        o.seed = seed;
        o.stream = 0x43544449u; // "CTDI": a stream word no patient run uses by default
        dxmcg_stats st {};
        rc = dxmcg_transport_run(g.w, &c, &o, nullptr, &st);
        if (rc != DXMCG_OK) {
            err = std::string("CTDI phantom run: ") + dxmcg_last_error();
            return rc;
        }
        std::vector<double> e(N);
        rc = dxmcg_world_read_tally(g.w, e.data(), nullptr, nullptr);
        if (rc != DXMCG_OK) {
            err = "CTDI phantom readout failed";
            return rc;
        }
        double energy[5] = {}, mass[5] = {};
        const double vol = sxy * sxy * sz;
        for (size_t v = 0; v < N; ++v)
            if (region[v] >= 0) {
                energy[region[v]] += e[v];
                mass[region[v]] += dens[v] * vol;
            }
        double ctdi100[5];
        for (int r = 0; r < 5; ++r)
            ctdi100[r] = (mass[r] > 0 ? energy[r] * kKeVToMilliGrayGram / mass[r] : 0.0) * 10.0 / b.collimation_cm;
        const double w = ctdi100[0] / 3.0 + (2.0 / 3.0) * 0.25 * (ctdi100[1] + ctdi100[2] + ctdi100[3] + ctdi100[4]);
        if (!(w > 0) || st.n_histories == 0) {
            err = "CTDI phantom: no dose scored";
            return DXMCG_ERR_DEVICE;
        }
        out = w / static_cast<double>(st.n_histories);
        return DXMCG_OK;
    }
} // namespace

double airKermaPerHistory(const dxmcg_beam& b)
{
    return b.energy_kev * airEnergyAbsorption(b.energy_kev) * kKeVToMilliGrayGram;
}

double dapPerHistory(const dxmcg_beam& b)
{
    const auto s = tubeSpectrum(b.kvp, b.anode_angle_deg, b.n_filters, b.filter_Z, b.filter_mm);
    double v = 0;
    for (size_t k = 0; k < s.energy.size(); ++k)
        v += s.weight[k] * s.energy[k] * airEnergyAbsorption(s.energy[k]);
    return v * kKeVToMilliGrayGram;
}

int calibrationFactor(const dxmcg_beam& b, int correction, const dxmcg_run_options& o, uint64_t nHist,
    bool allowPhantom, double& F, std::string& err)
{
    F = 1.0;
    if (!o.normalize)
        return DXMCG_OK;
    if (b.type == DXMCG_BEAM_DX || b.type == DXMCG_BEAM_CBCT) {
        if (b.dap_mgycm2 > 0) {
            const double per = dapPerHistory(b);
            if (!(per > 0) || nHist == 0) {
                err = "calibration: empty spectrum";
                return DXMCG_ERR_ARGUMENT;
            }
            F = b.dap_mgycm2 / (static_cast<double>(nHist) * per);
        }
        return DXMCG_OK;
    }
    if (b.type == DXMCG_BEAM_PENCIL) {
        if (b.air_kerma_mgy > 0) {
            const double per = airKermaPerHistory(b);
            if (!(per > 0) || nHist == 0) {
                err = "calibration: pencil energy out of range";
                return DXMCG_ERR_ARGUMENT;
            }
            F = b.air_kerma_mgy / (static_cast<double>(nHist) * per);
        }
        return DXMCG_OK;
    }
    if (!isCt(b.type))
        return DXMCG_OK;
    double target = b.ctdi_w_mgy;
    if (b.ctdi_vol_mgy > 0) {
        if (b.type == DXMCG_BEAM_CT_SEQUENTIAL)
            target = b.ctdi_vol_mgy * (b.slice_spacing_cm > 0 ? b.slice_spacing_cm / b.collimation_cm : 1.0);
        else
            target = b.ctdi_vol_mgy * b.pitch;
    }
    if (!(target > 0))
        return DXMCG_OK;
    if (!allowPhantom) {
        err = "calibration: CTDI normalisation simulates a phantom world and needs device allocations";
        return DXMCG_ERR_ARGUMENT;
    }
    double perHistory = 0;
    const int rc = ctdiwPerHistory(b, correction, o.seed, perHistory, err);
    if (rc != DXMCG_OK)
        return rc;
    const double perRotation = static_cast<double>(b.particles_per_exposure) * static_cast<double>(viewsPerRotation(b))
        * (b.type == DXMCG_BEAM_CT_SPIRAL_DUAL_ENERGY ? 2.0 : 1.0);
    F = target / (perHistory * perRotation);
    return DXMCG_OK;
}

} // namespace dxmcg
