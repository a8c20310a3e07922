// physics_engine.h / run_simulation.h - the transport driver of the MIDSX C++ API
// (reference: include/MIDSX/Core/physics_engine.h, run_simulation.h).
//
// runSimulation keeps the reference's signature (include/MIDSX/Core/run_simulation.h:24-27)
// and runs the history loop on the GPU through the C ABI: the tally factories are called
// once (the device accumulates atomically instead of per-thread replicas), the tables,
// phantom and source are uploaded once per engine and stay resident, and the results are
// written back into the tallies' quantity containers and, after
// addVoxelDataToComputationalDomain(), into the voxels' dose values.  Results of repeated
// runSimulation calls on one engine add up.
#pragma once
#include <cstdint>
#include <functional>
#include <memory>
#include <vector>

#include "../../midsx_gpu.h"
#include "computational_domain.h"
#include "source.h"
#include "surface_tally.h"
#include "volume_tally.h"

class PhysicsEngine {
public:
    PhysicsEngine(ComputationalDomain& comp_domain, InteractionData& interaction_data);
    ~PhysicsEngine();
    PhysicsEngine(const PhysicsEngine&) = delete;
    PhysicsEngine& operator=(const PhysicsEngine&) = delete;

    void addVolumeTallies(std::vector<std::unique_ptr<VolumeTally>>&& volume_tallies);
    void addSurfaceTallies(std::vector<std::unique_ptr<SurfaceTally>>&& surface_tallies);
    std::vector<VolumeQuantityContainer> getVolumeQuantityContainers();
    std::vector<SurfaceQuantityContainer> getSurfaceQuantityContainers();
    // Binned surface tallies (BinnedRectangularSurfaceTally) in the order they were added.
    std::vector<BinnedRectangularSurfaceTally*> getBinnedSurfaceTallies();
    void addVoxelDataToComputationalDomain();

    // GPU options (not in the reference): precision of the kernel, random seed and the
    // first history id of the next run.  The default is the plain FP64 form, the drop-in for
    // the reference's double-precision transport; MIDSX_PREC_MIXED (FP32 transport, 64-bit
    // fixed-point tallies) is opt-in.
    void setPrecision(midsx_precision p) { precision_ = p; }
    void setSeed(uint64_t seed) { seed_ = seed; }
    // Opt-in flight sampling (midsx_tracking; the reference's global-majorant Woodcock
    // tracking by default) and the macro-cell edge of MIDSX_TRACK_MACRO_CELL (a power of two,
    // 1..64 voxels; applied at the next run).
    void setTracking(midsx_tracking t) { tracking_ = t; }
    void setMacroCellEdge(int edge) { macro_edge_ = edge; }
    uint64_t nextHistoryId() const { return next_history_; }
    // Transports n histories from `source` into the engine's tallies.  Used by runSimulation.
    double run(PhotonSource& source, uint64_t n_photons);
    const midsx_run_stats& lastStats() const { return stats_; }

private:
    struct Device;
    ComputationalDomain& comp_domain_;
    InteractionData& interaction_data_;
    std::vector<std::unique_ptr<VolumeTally>> volume_tallies_;
    std::vector<std::unique_ptr<SurfaceTally>> surface_tallies_;
    std::unique_ptr<Device> dev_;
    midsx_precision precision_ = MIDSX_PREC_FP64;
    midsx_tracking tracking_ = MIDSX_TRACK_REFERENCE;
    int macro_edge_ = 0;  // 0: the phantom's own (MIDSX_MACRO_CELL)
    int macro_edge_applied_ = 0;
    uint64_t seed_ = 1;
    uint64_t next_history_ = 0;
    midsx_run_stats stats_{};
    std::vector<double> dose_sum_, dose_sumsq_, dose_count_;
    bool dose_pending_ = false;
    void ensureDevice(const midsx_source_spec& first_source);
};

void runSimulation(PhotonSource& source, PhysicsEngine& physics_engine,
                   std::function<std::vector<std::unique_ptr<SurfaceTally>>()> surface_tally_init,
                   std::function<std::vector<std::unique_ptr<VolumeTally>>()> volume_tally_init, int N_photons,
                   double& run_time);
void runSimulation(PhotonSource& source, PhysicsEngine& physics_engine,
                   std::function<std::vector<std::unique_ptr<SurfaceTally>>()> surface_tally_init,
                   std::function<std::vector<std::unique_ptr<VolumeTally>>()> volume_tally_init, int N_photons);
