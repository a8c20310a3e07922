// core_engine.cpp - PhysicsEngine and runSimulation of the MIDSX C++ API on the GPU.
// Reference: src/MIDSX/Core/physics_engine.cpp:11-168, src/MIDSX/Core/run_simulation.cpp:6-41.
// The history loop itself runs in the transport kernel behind the C ABI; this file moves
// the API objects to the device once, launches, and writes the device sums back into the
// reference's result objects.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

#include "MIDSX/Core/physics_engine.h"

namespace {
void check(midsx_status s, const char* what) {
    if (s == MIDSX_OK) return;
    std::string msg = std::string(what) + ": " + midsx_status_string(s) + " (" + midsx_last_error() + ")";
    if (s == MIDSX_NOT_FOUND) throw std::out_of_range(msg);
    if (s == MIDSX_INVALID_ARG) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

// Spectrum bins centred on a source's energies: one bin per line of a spectrum on an even
// grid (the reference's CSV spectra), a 1 eV bin around a single energy.  Lines off the grid
// of the smallest spacing still land in the bin that holds them.
void default_energy_bins(const midsx_source_spec& src, midsx_tally_spec& s) {
    if (src.spectrum_kind != MIDSX_SPEC_POLY || src.n_bins < 2 || !src.bin_energy) {
        const double e = src.spectrum_kind == MIDSX_SPEC_POLY && src.n_bins == 1 && src.bin_energy
                             ? src.bin_energy[0] : src.mono_energy;
        s.n_energy = 1;
        s.e_width = 1.0;
        s.e_min = e - 0.5;
        return;
    }
    std::vector<double> e(src.bin_energy, src.bin_energy + src.n_bins);
    std::sort(e.begin(), e.end());
    double step = 0;
    for (size_t i = 1; i < e.size(); ++i) {
        const double d = e[i] - e[i - 1];
        if (d > 0 && (step == 0 || d < step)) step = d;
    }
    if (step == 0) step = 1.0;
    const double span = (e.back() - e.front()) / step;
    s.e_width = step;
    s.e_min = e.front() - 0.5 * step;
    s.n_energy = int(std::min<double>(MIDSX_MAX_ENERGY_BINS, std::floor(span + 0.5) + 1));
}

}  // namespace

struct PhysicsEngine::Device {
    midsx_tables_h tables = nullptr;
    midsx_phantom_h phantom = nullptr;
    midsx_tallies_h tallies = nullptr;
    std::vector<int> spec_kind;
    std::vector<midsx_tally_spec> specs;
    ~Device() {
        if (tallies) midsx_gpu_tallies_destroy(tallies);
        if (phantom) midsx_gpu_phantom_destroy(phantom);
        if (tables) midsx_gpu_tables_destroy(tables);
    }
};

PhysicsEngine::PhysicsEngine(ComputationalDomain& comp_domain, InteractionData& interaction_data)
    : comp_domain_(comp_domain), interaction_data_(interaction_data) {}

PhysicsEngine::~PhysicsEngine() = default;

void PhysicsEngine::addVolumeTallies(std::vector<std::unique_ptr<VolumeTally>>&& v) {
    if (dev_) throw std::logic_error("tallies cannot be added after the first run of this engine");
    for (auto& t : v) volume_tallies_.push_back(std::move(t));
}

void PhysicsEngine::addSurfaceTallies(std::vector<std::unique_ptr<SurfaceTally>>&& s) {
    if (dev_) throw std::logic_error("tallies cannot be added after the first run of this engine");
    for (auto& t : s) surface_tallies_.push_back(std::move(t));
}

void PhysicsEngine::ensureDevice(const midsx_source_spec& first_source) {
    if (dev_) return;
    if (!interaction_data_.blob()) throw std::invalid_argument("InteractionData has no materials");
    const int n_grids = comp_domain_.getNumVoxelGrids();
    if (n_grids < 1 || n_grids > MIDSX_MAX_GRIDS)
        throw std::invalid_argument("the GPU transport takes a ComputationalDomain with 1 to 16 voxel grids");
    auto d = std::make_unique<Device>();
    check(midsx_gpu_tables_create(interaction_data_.blob(), &d->tables), "midsx_gpu_tables_create");
    // every grid, in the domain's order (getVoxel's first-hit order)
    std::vector<std::vector<uint8_t>> ids(static_cast<size_t>(n_grids));
    std::vector<midsx_grid_spec> grids(static_cast<size_t>(n_grids));
    for (int k = 0; k < n_grids; ++k) {
        VoxelGrid& g = comp_domain_.getVoxelGridN(k);
        midsx_grid_spec& gs = grids[size_t(k)];
        std::memset(&gs, 0, sizeof(gs));
        const Vec3 org = comp_domain_.getVoxelGridOriginN(k), sp = g.getSpacing();
        const VoxelIndex dims = g.getDimVox();
        for (int i = 0; i < 3; ++i) {
            gs.origin[i] = org(i);
            gs.spacing[i] = sp(i);
            gs.dims[i] = dims[size_t(i)];
        }
        ids[size_t(k)] = g.getMaterialIdArray();
        gs.ids = ids[size_t(k)].data();
    }
    const Vec3 dom = comp_domain_.getDimSpace();
    const double domain[3] = {dom(0), dom(1), dom(2)};
    check(midsx_gpu_phantom_create_grids(d->tables, domain, comp_domain_.background_voxel.materialID, grids.data(),
                                         n_grids, &d->phantom),
          "midsx_gpu_phantom_create_grids");
    std::vector<midsx_tally_spec> specs;
    for (auto& t : surface_tallies_) {
        midsx_tally_spec s = t->describe();
        // a disc or rectangle measuring IncidentEnergy keeps a spectrum for DerivedQuantity
        if (s.kind != MIDSX_TALLY_SURFACE_BINNED_RECT && !t->hasEnergyBins() &&
            t->getSurfaceQuantityContainer().getVectorQuantities().count(VectorSurfaceQuantityType::IncidentEnergy))
            default_energy_bins(first_source, s);
        specs.push_back(s);
    }
    for (auto& t : volume_tallies_) specs.push_back(t->describe());
    for (auto& s : specs) d->spec_kind.push_back(s.kind);
    d->specs = specs;
    check(midsx_gpu_tallies_create(d->phantom, specs.data(), int32_t(specs.size()), MIDSX_DOSE_FULL, &d->tallies),
          "midsx_gpu_tallies_create");
    dev_ = std::move(d);
}

double PhysicsEngine::run(PhotonSource& source, uint64_t n_photons) {
    midsx_source_spec spec = source.describe();
    ensureDevice(spec);
    if (macro_edge_ != 0 && macro_edge_ != macro_edge_applied_) {
        check(midsx_gpu_phantom_macro_cells(dev_->phantom, macro_edge_), "midsx_gpu_phantom_macro_cells");
        macro_edge_applied_ = macro_edge_;
    }
    midsx_source_h src = nullptr;
    check(midsx_gpu_source_create(&spec, &src), "midsx_gpu_source_create");
    midsx_run_config cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.precision = precision_;
    cfg.tracking = tracking_;
    cfg.seed = seed_;
    cfg.first_history = next_history_;
    cfg.n_histories = n_photons;
    auto t0 = std::chrono::steady_clock::now();
    midsx_status st = midsx_gpu_run(dev_->tables, dev_->phantom, src, dev_->tallies, &cfg, nullptr);
    if (st == MIDSX_OK) st = midsx_gpu_fetch_stats(dev_->tallies, &stats_, nullptr);
    double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    midsx_gpu_source_destroy(src);
    // a history that reached the step or Compton-trial cap was cut short, which the reference's
    // unbounded loop never does: the run's results would be biased, so it is an error (the
    // counts stay in lastStats())
    check(st, "midsx_gpu_run");
    next_history_ += n_photons;
    // scalar and binned tallies: the device holds cumulative sums over all runs
    size_t k = 0;
    double slots[MIDSX_SCALAR_SLOTS];
    for (auto& t : surface_tallies_) {
        const int kind = dev_->spec_kind[k];
        if (kind == MIDSX_TALLY_SURFACE_BINNED_RECT) {
            auto* b = static_cast<BinnedRectangularSurfaceTally*>(t.get());
            check(midsx_gpu_fetch_binned(dev_->tallies, int32_t(k), b->energies().data(), b->counts().data(), nullptr),
                  "midsx_gpu_fetch_binned");
        } else {
            check(midsx_gpu_fetch_scalar(dev_->tallies, int32_t(k), slots, nullptr), "midsx_gpu_fetch_scalar");
            SurfaceQuantityContainer& c = t->getSurfaceQuantityContainer();
            for (auto& q : c.getVectorQuantities()) {
                int qi = q.first == VectorSurfaceQuantityType::IncidentEnergy ? 0 : 1;
                for (int cls = 0; cls < 4; ++cls) {
                    VectorValue v;
                    const double* s = slots + qi * 12 + cls * 3;
                    v.addSummary(s[0], s[1], s[2]);
                    q.second.getClassValues(cls) = v;
                }
            }
            for (auto& q : c.getCountQuantities())
                for (int cls = 0; cls < 4; ++cls) q.second.getClassValues(cls).count_ = (long long)slots[24 + cls];
            const midsx_tally_spec& ts = dev_->specs[k];
            if (ts.n_energy > 0) {
                IncidentSpectrum& sp = c.getIncidentSpectrum();
                sp.e_min = ts.e_min;
                sp.e_width = ts.e_width;
                sp.n = ts.n_energy;
                sp.count.assign(size_t(ts.n_energy) * 4, 0.0);
                sp.cosine.assign(size_t(ts.n_energy) * 4, 0.0);
                check(midsx_gpu_fetch_spectrum(dev_->tallies, int32_t(k), sp.count.data(), sp.cosine.data(), nullptr),
                      "midsx_gpu_fetch_spectrum");
            }
        }
        ++k;
    }
    for (auto& t : volume_tallies_) {
        check(midsx_gpu_fetch_scalar(dev_->tallies, int32_t(k), slots, nullptr), "midsx_gpu_fetch_scalar");
        VolumeQuantityContainer& c = t->getVolumeQuantityContainer();
        for (auto& q : c.getVectorQuantities()) {
            int qi = q.first == VectorVolumeQuantityType::EnergyDeposition ? 0 : 1;
            for (int cls = 0; cls < 4; ++cls) {
                VectorValue v;
                const double* s = slots + qi * 12 + cls * 3;
                v.addSummary(s[0], s[1], s[2]);
                q.second.getClassValues(cls) = v;
            }
        }
        for (auto& q : c.getCountQuantities()) {
            int base = q.first == CountVolumeQuantityType::NumberOfPhotons ? 24 : 28;
            for (int cls = 0; cls < 4; ++cls) q.second.getClassValues(cls).count_ = (long long)slots[base + cls];
        }
        ++k;
    }
    size_t nv = 0;
    for (int k = 0; k < comp_domain_.getNumVoxelGrids(); ++k) nv += comp_domain_.getVoxelGridN(k).getNumberOfVoxels();
    dose_sum_.resize(nv);
    dose_sumsq_.resize(nv);
    dose_count_.resize(nv);
    check(midsx_gpu_fetch_dose(dev_->tallies, dose_sum_.data(), dose_sumsq_.data(), dose_count_.data(), nullptr),
          "midsx_gpu_fetch_dose");
    dose_pending_ = true;
    return seconds;
}

std::vector<VolumeQuantityContainer> PhysicsEngine::getVolumeQuantityContainers() {
    std::vector<VolumeQuantityContainer> out;
    for (auto& t : volume_tallies_) out.push_back(t->getVolumeQuantityContainer());
    return out;
}

std::vector<SurfaceQuantityContainer> PhysicsEngine::getSurfaceQuantityContainers() {
    std::vector<SurfaceQuantityContainer> out;
    for (auto& t : surface_tallies_)
        if (!dynamic_cast<BinnedRectangularSurfaceTally*>(t.get())) out.push_back(t->getSurfaceQuantityContainer());
    return out;
}

std::vector<BinnedRectangularSurfaceTally*> PhysicsEngine::getBinnedSurfaceTallies() {
    std::vector<BinnedRectangularSurfaceTally*> out;
    for (auto& t : surface_tallies_)
        if (auto* b = dynamic_cast<BinnedRectangularSurfaceTally*>(t.get())) out.push_back(b);
    return out;
}

void PhysicsEngine::addVoxelDataToComputationalDomain() {
    if (!dose_pending_) return;
    // the device numbers voxels grid after grid
    size_t off = 0;
    for (int k = 0; k < comp_domain_.getNumVoxelGrids(); ++k) {
        std::vector<Voxel>& vox = comp_domain_.getVoxelGridN(k).voxels();
        for (size_t i = 0; i < vox.size(); ++i) {
            VectorValue v;
            v.addSummary(dose_count_[off + i], dose_sum_[off + i], dose_sumsq_[off + i]);
            vox[i].dose = v;
        }
        off += vox.size();
    }
    dose_pending_ = false;
}

void runSimulation(PhotonSource& source, PhysicsEngine& physics_engine,
                   std::function<std::vector<std::unique_ptr<SurfaceTally>>()> surface_tally_init,
                   std::function<std::vector<std::unique_ptr<VolumeTally>>()> volume_tally_init, int N_photons,
                   double& run_time) {
    if (N_photons < 0) throw std::invalid_argument("N_photons must be non-negative");
    if (physics_engine.nextHistoryId() == 0) {
        physics_engine.addSurfaceTallies(surface_tally_init());
        physics_engine.addVolumeTallies(volume_tally_init());
    }
    run_time = physics_engine.run(source, uint64_t(N_photons));
    physics_engine.addVoxelDataToComputationalDomain();
}

void runSimulation(PhotonSource& source, PhysicsEngine& physics_engine,
                   std::function<std::vector<std::unique_ptr<SurfaceTally>>()> surface_tally_init,
                   std::function<std::vector<std::unique_ptr<VolumeTally>>()> volume_tally_init, int N_photons) {
    double t = 0;
    runSimulation(source, physics_engine, std::move(surface_tally_init), std::move(volume_tally_init), N_photons, t);
}
