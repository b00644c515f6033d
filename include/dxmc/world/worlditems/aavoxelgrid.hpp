// dxmc/world/worlditems/aavoxelgrid.hpp -- axis-aligned voxel grid item:
// setData(dims, density, material index, materials), setSpacing (cm), build, and the
// per-voxel doseScored(i).dose()/variance()/numberOfEvents() readback
// (simulationpipeline.cpp:127-153, :174-231).  The grid lives on the GPU after
// build(); the dose arrays are copied back once after each transport, on the first
// doseScored() call.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../dxmcg.h"

namespace dxmc {

class DoseScore {
public:
    DoseScore() = default;
    DoseScore(double dose, double variance, std::uint64_t events)
        : m_dose(dose)
        , m_var(variance)
        , m_events(events)
    {
    }
    double dose() const { return m_dose; }
    double variance() const { return m_var; }
    double standardDeviation() const { return std::sqrt(m_var); }
    double relativeUncertainty() const { return m_dose > 0 ? std::sqrt(m_var) / m_dose : 0.0; }
    std::uint64_t numberOfEvents() const { return m_events; }

private:
    double m_dose = 0;
    double m_var = 0;
    std::uint64_t m_events = 0;
};

template <int NMaterialShells = 5, int LOWENERGYCORRECTION = 2, int TRANSPARENTVOXELS = 255>
class AAVoxelGrid {
public:
    AAVoxelGrid() = default;
    AAVoxelGrid(const AAVoxelGrid&) = delete;
    AAVoxelGrid& operator=(const AAVoxelGrid&) = delete;
    ~AAVoxelGrid() { dxmcg_world_destroy(m_world); }

    // Returns false if the arrays do not match dims or a composition is invalid.
    template <typename MaterialT>
    bool setData(const std::array<std::size_t, 3>& dims, const std::vector<double>& density,
        const std::vector<std::uint8_t>& materialIdx, const std::vector<MaterialT>& materials)
    {
        const std::size_t n = dims[0] * dims[1] * dims[2];
        if (n == 0 || density.size() != n || materialIdx.size() != n || materials.empty()
            || materials.size() > DXMCG_MAX_MATERIALS)
            return false;
        m_dims = dims;
        m_density = density;
        m_material = materialIdx;
        m_materials.clear();
        for (const auto& m : materials)
            m_materials.push_back(m.composition());
        m_built = false;
        return true;
    }
    void setSpacing(const std::array<double, 3>& cm)
    {
        m_spacing = cm;
        m_built = false;
    }
    const std::array<double, 3>& spacing() const { return m_spacing; }
    const std::array<std::size_t, 3>& dimensions() const { return m_dims; }
    std::size_t size() const { return m_dims[0] * m_dims[1] * m_dims[2]; }
    std::array<double, 6> AABB() const
    {
        std::array<double, 6> a {};
        for (int i = 0; i < 3; ++i) {
            a[i] = -0.5 * m_dims[i] * m_spacing[i];
            a[i + 3] = 0.5 * m_dims[i] * m_spacing[i];
        }
        return a;
    }

    // World::build(): the grid moves to the GPU (throws std::runtime_error on failure)
    void build()
    {
        if (m_built)
            return;
        dxmcg_world_destroy(m_world);
        m_world = nullptr;
        const int32_t dims[3] = { static_cast<int32_t>(m_dims[0]), static_cast<int32_t>(m_dims[1]),
            static_cast<int32_t>(m_dims[2]) };
        int rc = dxmcg_world_create(dims, m_spacing.data(), m_materials.data(), static_cast<int>(m_materials.size()),
            LOWENERGYCORRECTION, &m_world);
        if (rc == DXMCG_OK)
            rc = dxmcg_world_set_data(m_world, m_density.data(), m_material.data());
        if (rc == DXMCG_OK)
            rc = dxmcg_world_build(m_world);
        if (rc != DXMCG_OK)
            throw std::runtime_error(std::string("AAVoxelGrid::build: ") + dxmcg_last_error());
        m_density.clear();
        m_density.shrink_to_fit();
        m_material.clear();
        m_material.shrink_to_fit();
        m_scores.clear();
        m_built = true;
    }

    const DoseScore& doseScored(std::size_t i) const
    {
        if (m_stale || m_scores.size() != size())
            readBack();
        return m_scores[i];
    }
    void clearDoseScored()
    {
        if (m_world)
            dxmcg_world_clear_tally(m_world);
        m_scores.clear();
        m_stale = true;
    }

    dxmcg_world* engineWorld() const { return m_world; }
    void transported() { m_stale = true; }

private:
    void readBack() const
    {
        const std::size_t n = size();
        std::vector<double> d(n), v(n);
        std::vector<std::uint64_t> c(n);
        if (!m_world || dxmcg_world_read_dose(m_world, d.data(), v.data(), c.data()) != DXMCG_OK)
            std::fill(d.begin(), d.end(), 0.0);
        m_scores.resize(n);
        for (std::size_t i = 0; i < n; ++i)
            m_scores[i] = DoseScore(d[i], v[i], c[i]);
        m_stale = false;
    }

    std::array<std::size_t, 3> m_dims { 1, 1, 1 };
    std::array<double, 3> m_spacing { 1, 1, 1 };
    std::vector<double> m_density;
    std::vector<std::uint8_t> m_material;
    std::vector<dxmcg_material> m_materials;
    dxmcg_world* m_world = nullptr;
    bool m_built = false;
    mutable bool m_stale = true;
    mutable std::vector<DoseScore> m_scores;
};

} // namespace dxmc
