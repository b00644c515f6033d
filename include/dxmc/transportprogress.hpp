// dxmc/transportprogress.hpp -- progress and cooperative stop shared between the
// thread running the transport and the GUI thread: progress() -> (done, total),
// message(), continueSimulation(), setStopSimulation()
// (simulationpipeline.cpp:114-120, :169, :234, :261).  Thread-safe.
#pragma once

#include <cstdint>
#include <string>
#include <utility>

#include "../dxmcg.h"

namespace dxmc {

class TransportProgress {
public:
    TransportProgress()
        : m_p(dxmcg_progress_create())
    {
    }
    TransportProgress(const TransportProgress&) = delete;
    TransportProgress& operator=(const TransportProgress&) = delete;
    ~TransportProgress() { dxmcg_progress_destroy(m_p); }

    std::pair<std::uint64_t, std::uint64_t> progress() const
    {
        std::uint64_t done = 0, total = 1;
        dxmcg_progress_get(m_p, &done, &total);
        return { done, total };
    }
    std::string message() const
    {
        char buf[256];
        dxmcg_progress_message(m_p, buf, sizeof(buf));
        return std::string(buf);
    }
    bool continueSimulation() const { return dxmcg_progress_continue(m_p) != 0; }
    void setStopSimulation() { dxmcg_progress_stop(m_p); }
    // a new transport starts: clears a stop request left by the previous simulation
    void start() { dxmcg_progress_reset(m_p); }

    dxmcg_progress* handle() const { return m_p; }

private:
    dxmcg_progress* m_p;
};

} // namespace dxmc
