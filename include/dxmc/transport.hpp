// dxmc/transport.hpp -- Transport: runs one beam through every voxel grid of a
// world on the GPU (transport(world, beam, progress, true),
// simulationpipeline.cpp:155-171).  The trailing bool asks for the beam's dose
// calibration (DAP for DX/CBCT, CTDIvol/CTDIw for CT).  Each call uses its own
// random stream (seed, call number); setNumberOfThreads is accepted and has no
// effect (the whole GPU is used).
#pragma once

#include <cstdint>
#include <string>

#include "../dxmcg.h"
#include "transportprogress.hpp"

namespace dxmc {

class Transport {
public:
    void setNumberOfThreads(std::uint64_t) { }
    std::uint64_t numberOfThreads() const { return 1; }
    void setSeed(std::uint64_t seed) { m_seed = seed; }
    std::uint64_t seed() const { return m_seed; }
    void setTracking(int tracking) { m_tracking = tracking; }

    template <typename W, typename B>
    void operator()(W& world, const B& beam, TransportProgress* progress = nullptr, bool useBeamCalibration = true)
    {
        const dxmcg_beam d = beam.descriptor();
        dxmcg_run_options o {};
        o.seed = m_seed;
        o.stream = m_calls++;
        o.tracking = m_tracking;
        o.normalize = useBeamCalibration ? 1 : 0;
        if (progress)
            progress->start();
        m_status = DXMCG_OK;
        world.forEachItem([&](auto& grid) {
            if (m_status != DXMCG_OK)
                return;
            m_status = dxmcg_transport_run(grid.engineWorld(), &d, &o, progress ? progress->handle() : nullptr,
                &m_stats);
            grid.transported();
            if (m_status != DXMCG_OK && m_status != DXMCG_ERR_CANCELLED)
                m_error = dxmcg_last_error();
        });
    }

    // status and statistics of the last call (DXMCG_OK, DXMCG_ERR_CANCELLED, ...)
    int lastStatus() const { return m_status; }
    const std::string& lastError() const { return m_error; }
    const dxmcg_stats& lastStats() const { return m_stats; }

private:
    std::uint64_t m_seed = 1;
    std::uint32_t m_calls = 0;
    int m_tracking = DXMCG_TRACK_WOODCOCK;
    int m_status = DXMCG_OK;
    std::string m_error;
    dxmcg_stats m_stats {};
};

} // namespace dxmc
