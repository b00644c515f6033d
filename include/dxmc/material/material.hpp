// dxmc/material/material.hpp -- Material<N>: composition by mass and its photon
// attenuation (Material::byWeight, simulationpipeline.cpp:136;
// attenuationValues(E).sum(), ctsegmentationpipeline.cpp:84-104), on the engine's
// host physics (dxmcg_material_attenuation).  N (the number of electron shells the
// reference keeps) is accepted for source compatibility; the engine's model has
// no per-shell data.
#pragma once

#include <cstdint>
#include <map>
#include <optional>
#include <string>

#include "../../dxmcg.h"

namespace dxmc {

namespace detail {
    // Named materials the layer knows (see nistmaterials.hpp): by mass, from the
    // chemical formula (water, PMMA) or the usual dry-air fractions.
    inline std::optional<std::map<std::size_t, double>> namedComposition(const std::string& name)
    {
        if (name == "Water, Liquid")
            return std::map<std::size_t, double> { { 1, 11.19 }, { 8, 88.81 } };
        if (name == "Air, Dry (near sea level)")
            return std::map<std::size_t, double> { { 7, 75.5 }, { 8, 23.2 }, { 18, 1.3 } };
        if (name == "Polymethyl Methacralate (Lucite, Perspex)")
            return std::map<std::size_t, double> { { 1, 8.054 }, { 6, 59.985 }, { 8, 31.961 } };
        return std::nullopt;
    }
} // namespace detail

template <typename T = double>
struct AttenuationValues {
    T photoelectric = 0;
    T incoherent = 0;
    T coherent = 0;
    T sum() const { return photoelectric + incoherent + coherent; }
};

template <std::size_t NMaterialShells = 5, int LOWENERGYCORRECTION = 1>
class Material {
public:
    // mass fractions by atomic number; std::nullopt for an empty or invalid composition
    template <typename MapT>
    static std::optional<Material> byWeight(const MapT& Z_by_weight)
    {
        Material m;
        m.m_mat = dxmcg_material {};
        for (const auto& [Z, w] : Z_by_weight) {
            if (w <= 0)
                continue;
            if (m.m_mat.n >= DXMCG_MAX_ELEMENTS || Z < 1 || Z > 92)
                return std::nullopt;
            m.m_mat.Z[m.m_mat.n] = static_cast<int32_t>(Z);
            m.m_mat.w[m.m_mat.n] = static_cast<double>(w);
            ++m.m_mat.n;
        }
        if (m.m_mat.n == 0)
            return std::nullopt;
        const double E = 60.0;
        double a, b, c;
        if (dxmcg_material_attenuation(&m.m_mat, 1, 1, &E, &a, &b, &c) != DXMCG_OK)
            return std::nullopt;
        return m;
    }

    static std::optional<Material> byNistName(const std::string& name)
    {
        const auto c = detail::namedComposition(name);
        if (!c)
            return std::nullopt;
        return byWeight(*c);
    }

    AttenuationValues<double> attenuationValues(double energy_kev) const
    {
        AttenuationValues<double> v;
        dxmcg_material_attenuation(&m_mat, LOWENERGYCORRECTION, 1, &energy_kev, &v.photoelectric, &v.incoherent,
            &v.coherent);
        return v;
    }

    const dxmcg_material& composition() const { return m_mat; }

private:
    dxmcg_material m_mat {};
};

} // namespace dxmc
