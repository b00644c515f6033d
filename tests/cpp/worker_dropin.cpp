// The call sequence of OpenDXMC's SimulationPipeline worker
// (src/libopendxmc/simulationpipeline.cpp:124-235) written against the dxmc:: layer
// over the GB300 engine: materials by weight, AAVoxelGrid::setData/setSpacing,
// World::build, Transport over two beams with a shared TransportProgress, then the
// per-voxel doseScored(i) readback.  Used by tests/test_gpu_dropin.py.
//
// usage: worker_dropin <nx> <ny> <nz> <sx> <sy> <sz> density.f64 material.u8 out.bin
// out.bin: N doubles dose, N doubles variance, N uint64 events (both beams summed)
#include <array>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <map>
#include <vector>

#include "dxmc/beams/ctspiralbeam.hpp"
#include "dxmc/beams/dxbeam.hpp"
#include "dxmc/material/material.hpp"
#include "dxmc/transport.hpp"
#include "dxmc/transportprogress.hpp"
#include "dxmc/world/world.hpp"
#include "dxmc/world/worlditems/aavoxelgrid.hpp"

using Material = dxmc::Material<5>;
using VoxelGrid = dxmc::AAVoxelGrid<5, 1, 255>;
using World = dxmc::World<VoxelGrid>;

template <typename T>
static std::vector<T> readFile(const char* path, std::size_t n)
{
    std::vector<T> v(n);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * sizeof(T)));
    return v;
}

int main(int argc, char** argv)
{
    if (argc != 10) {
        std::fprintf(stderr, "usage: worker_dropin nx ny nz sx sy sz density material out\n");
        return 2;
    }
    const std::array<std::size_t, 3> dims = { std::stoul(argv[1]), std::stoul(argv[2]), std::stoul(argv[3]) };
    const std::array<double, 3> spacing = { std::stod(argv[4]), std::stod(argv[5]), std::stod(argv[6]) };
    const std::size_t N = dims[0] * dims[1] * dims[2];
    const auto density = readFile<double>(argv[7], N);
    const auto material = readFile<std::uint8_t>(argv[8], N);

    // materials by mass fraction, as DataContainer::Material carries them
    const std::vector<std::map<std::uint64_t, double>> templates = {
        { { 7, 80.0 }, { 8, 20.0 } }, { { 1, 11.2 }, { 8, 88.8 } },
        { { 1, 3.6 }, { 6, 15.9 }, { 7, 4.2 }, { 8, 44.8 }, { 11, 0.3 }, { 12, 0.2 }, { 15, 9.4 }, { 16, 0.3 }, { 20, 21.3 } }
    };
    World world;
    auto& vgrid = world.addItem<VoxelGrid>();
    {
        std::vector<Material> materials;
        for (const auto& t : templates) {
            auto m = Material::byWeight(t);
            if (!m)
                return 3;
            materials.push_back(m.value());
        }
        if (!vgrid.setData(dims, density, material, materials))
            return 4;
        vgrid.setSpacing(spacing);
    }
    world.build();

    dxmc::TransportProgress progress;
    dxmc::Transport transport;
    transport.setNumberOfThreads(16);

    // DX beam as OpenDXMC's DXBeam sets it up at 0/0 degrees (dxmc_specialization.cpp:21-90)
    dxmc::DXBeam<false> dx({ 0, 100, 0 }, { { { 0, 0, 1 }, { -1, 0, 0 } } }, { { 13, 2.5 } });
    dx.setTubeVoltage(70.0);
    dx.setCollimationHalfAngles({ std::tan(0.5 * 10.0 / 100.0), std::tan(0.5 * 10.0 / 100.0) });
    dx.setNumberOfExposures(4);
    dx.setNumberOfParticlesPerExposure(50000);
    dx.setDAPvalue(10.0);

    dxmc::CTSpiralBeam<false> ct({ 0, 0, -2 }, { 0, 0, 2 }, { { 13, 6.0 } });
    ct.setTubeVoltage(120.0);
    ct.setSourceDetectorDistance(119.0);
    ct.setCollimation(2.0);
    ct.setPitch(1.0);
    ct.setStepAngleDeg(10.0);
    ct.setScanFieldOfView(50.0);
    ct.setNumberOfParticlesPerExposure(2000);
    ct.setBowtieFilter(dxmc::BowtieFilter({ { 0.0, 1.88 }, { 0.0839, 1.49 }, { 0.167, 0.73 }, { 0.39, 0.30 } }));
    ct.setCTDIvol(5.0);

    transport(world, dx, &progress, true);
    if (transport.lastStatus() != DXMCG_OK || !progress.continueSimulation()) {
        std::fprintf(stderr, "dx transport failed: %s\n", transport.lastError().c_str());
        return 5;
    }
    transport(world, ct, &progress, true);
    if (transport.lastStatus() != DXMCG_OK) {
        std::fprintf(stderr, "ct transport failed: %s\n", transport.lastError().c_str());
        return 6;
    }
    const auto [done, total] = progress.progress();

    std::vector<double> dose(N), var(N);
    std::vector<std::uint64_t> count(N);
    for (std::size_t i = 0; i < N; ++i) {
        const auto& s = vgrid.doseScored(i);
        dose[i] = s.dose();
        var[i] = s.variance();
        count[i] = s.numberOfEvents();
    }
    std::ofstream out(argv[9], std::ios::binary);
    out.write(reinterpret_cast<const char*>(dose.data()), static_cast<std::streamsize>(N * sizeof(double)));
    out.write(reinterpret_cast<const char*>(var.data()), static_cast<std::streamsize>(N * sizeof(double)));
    out.write(reinterpret_cast<const char*>(count.data()), static_cast<std::streamsize>(N * sizeof(std::uint64_t)));
    std::printf("{\"exposures_dx\": %llu, \"exposures_ct\": %llu, \"progress\": [%llu, %llu], \"message\": \"%s\"}\n",
        static_cast<unsigned long long>(dx.numberOfExposures()), static_cast<unsigned long long>(ct.numberOfExposures()),
        static_cast<unsigned long long>(done), static_cast<unsigned long long>(total), progress.message().c_str());
    return 0;
}
