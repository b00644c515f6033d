// dxmc/beams/tube/tube.hpp -- X-ray tube: voltage, anode angle, filtration and the
// spectrum on 1 keV bins (Tube(kvp), setAlFiltration, setSnFiltration, getEnergy,
// getSpecter: ctsegmentationpipeline.cpp:66-71; filtration(Z): hdf5wrapper.cpp:483-485;
// beam-level setters: beamsettingsmodel.cpp:257-330), on the engine's host model
// (dxmcg_tube_spectrum: Kramers' law, tungsten K lines, exponential filtration).
#pragma once

#include <cstdint>
#include <map>
#include <vector>

#include "../../../dxmcg.h"

namespace dxmc {

class Tube {
public:
    Tube(double tubeVoltage = 120.0, double anodeAngleDeg = 12.0, double energyResolution = 1.0)
        : m_voltage(tubeVoltage)
        , m_anodeAngleDeg(anodeAngleDeg)
        , m_energyResolution(energyResolution)
    {
    }

    double voltage() const { return m_voltage; }
    void setVoltage(double kvp) { m_voltage = kvp; }
    double anodeAngleDeg() const { return m_anodeAngleDeg; }
    void setAnodeAngleDeg(double a) { m_anodeAngleDeg = a; }
    double energyResolution() const { return m_energyResolution; }
    void setEnergyResolution(double) { } // the engine's spectra are on 1 keV bins

    void addFiltrationMaterial(std::size_t Z, double mm)
    {
        if (mm > 0)
            m_filtration[Z] = mm;
        else
            m_filtration.erase(Z);
    }
    double filtration(std::size_t Z) const
    {
        const auto it = m_filtration.find(Z);
        return it == m_filtration.end() ? 0.0 : it->second;
    }
    const std::map<std::size_t, double>& filtrationMaterials() const { return m_filtration; }
    void clearFiltrationMaterials() { m_filtration.clear(); }
    void setAlFiltration(double mm) { addFiltrationMaterial(13, mm); }
    void setCuFiltration(double mm) { addFiltrationMaterial(29, mm); }
    void setSnFiltration(double mm) { addFiltrationMaterial(50, mm); }
    double AlFiltration() const { return filtration(13); }
    double CuFiltration() const { return filtration(29); }
    double SnFiltration() const { return filtration(50); }

    std::vector<double> getEnergy() const
    {
        std::vector<double> e, w;
        spectrum(e, w);
        return e;
    }

    // weights at the given energies (bins of 1 keV); normalised to sum 1 if asked
    std::vector<double> getSpecter(const std::vector<double>& energies, bool normalize = true) const
    {
        std::vector<double> e, w;
        spectrum(e, w);
        std::vector<double> out(energies.size(), 0.0);
        double s = 0;
        for (std::size_t i = 0; i < energies.size(); ++i) {
            const long k = static_cast<long>(energies[i] + 0.5) - 1;
            if (k >= 0 && k < static_cast<long>(w.size()))
                out[i] = w[k];
            s += out[i];
        }
        if (normalize && s > 0)
            for (auto& x : out)
                x /= s;
        return out;
    }

    double mmAlHalfValueLayer() const
    {
        int32_t Z[8];
        double mm[8];
        const int n = filters(Z, mm);
        double hvl = 0;
        dxmcg_tube_al_hvl(m_voltage, n, Z, mm, &hvl);
        return hvl;
    }

    double meanSpecterEnergy() const
    {
        int32_t Z[8];
        double mm[8];
        const int n = filters(Z, mm);
        double m = 0;
        dxmcg_tube_mean_energy(m_voltage, n, Z, mm, &m);
        return m;
    }

    // fills the engine's filter arrays (at most 8 materials)
    int filters(int32_t* Z, double* mm) const
    {
        int n = 0;
        for (const auto& [z, t] : m_filtration) {
            if (n == 8)
                break;
            Z[n] = static_cast<int32_t>(z);
            mm[n] = t;
            ++n;
        }
        return n;
    }

private:
    void spectrum(std::vector<double>& e, std::vector<double>& w) const
    {
        int32_t Z[8];
        double mm[8];
        const int n = filters(Z, mm);
        int count = 0;
        if (dxmcg_tube_spectrum(m_voltage, m_anodeAngleDeg, n, Z, mm, nullptr, nullptr, 0, &count) != DXMCG_OK)
            return;
        e.resize(count);
        w.resize(count);
        dxmcg_tube_spectrum(m_voltage, m_anodeAngleDeg, n, Z, mm, e.data(), w.data(), count, &count);
    }

    double m_voltage;
    double m_anodeAngleDeg;
    double m_energyResolution;
    std::map<std::size_t, double> m_filtration;
};

} // namespace dxmc
