// kernel_body.cuh - the transport kernel (included by transport.cu).
//
// Layout of the work: every lane of a warp owns one history at a time (history ids strided by
// the number of threads).  Each loop iteration is one Woodcock step
// (src/MIDSX/Core/physics_engine.cpp:28-79) for every lane that is flying.  The long, rare
// pieces of work are "events": a real collision (interaction type, Rayleigh / Compton /
// photoelectric sampling, tallies, dose) and the start of a new history (source sampling and
// the per-energy table lookups).  A lane that needs an event parks; the warp runs the parked
// events once `regroup` of its lanes wait - or no lane is left flying - so that event code
// runs with many lanes active instead of one (warp ballot; each interaction type is then a
// branch of its own).  Per-history counters stay in 32-bit registers and are flushed to
// shared-memory block counters when the history ends; one atomic per block and counter at
// the end.

// per-energy cache: majorant and every material's total cross section and delta-scatter
// threshold (isDeltaScatter: p_delta = 1 - mu / mu_max), kept per thread in shared memory
template <typename R>
__device__ __noinline__ R refresh_energy(const RunParams& P, R E, R* thr, R* mu, int stride) {
    R mu_max = lin_lookup<R>(P.T, P.T.majorant, E);
    for (int m = 0; m < P.T.n_materials; ++m) {
        R mm = lin_lookup<R>(P.T, P.T.mat[m].total, E);
        mu[m * stride] = mm;
        thr[m * stride] = R(1) - mm / mu_max;
    }
    return mu_max;
}

// Compton scattering by Kahn's method with the S(x) rejection
// (src/MIDSX/Core/photon_interactions.cpp:62-141).  Returns false at the trial cap.
template <typename R>
__device__ __noinline__ bool sample_compton(const RunParams& P, const DevMaterial& Mt, HistoryRng& rng, R E, R& mu,
                                            R& kp, uint32_t& trials) {
    const R alpha = R(P.T.alpha);
    const R k = E / R(kMec2);
    const R r1p = (R(1) + R(2) * k) / (R(9) + R(2) * k);
    const R s_max = lin_lookup<R>(P.T, Mt.sfunc, alpha * k * sqrt_(R(2)));
    for (int trial = 0; trial < P.max_trials; ++trial) {
        ++trials;
        R r1 = uniform<R>(rng), r2 = uniform<R>(rng), r3 = uniform<R>(rng);
        R chi;
        if (r1 <= r1p) {
            chi = R(1) + R(2) * k * r2;
            if (!(r3 <= R(4) * (R(1) / chi - R(1) / (chi * chi)))) continue;
        } else {
            chi = (R(1) + R(2) * k) / (R(1) + R(2) * k * r2);
            R tt = R(1) / k - chi / k + R(1);
            if (!(R(2) * r3 <= tt * tt + R(1) / chi)) continue;
        }
        kp = k / chi;
        mu = R(1) + R(1) / k - R(1) / kp;
        R x = alpha * k * sqrt_(R(1) - mu);
        R accept = lin_lookup<R>(P.T, Mt.sfunc, x) / s_max;
        if (uniform<R>(rng) <= accept) return true;
    }
    return false;
}

template <bool MX>
__device__ __noinline__ void score_dose(const RunParams& P, int vox, double dep) {
    unsigned long long* rec = P.dose + size_t(vox) * P.dose_stride;
    Acc<MX>::energy(rec, dep);
    if (P.dose_stride > 1) {
        Acc<MX>::energy2(rec + 1, dep);
        count1(rec + 2);
    }
}

__device__ __forceinline__ void stat_add(unsigned long long* s, int slot, unsigned long long v) {
    if (v) atomicAdd(s + slot, v);
}

__device__ __forceinline__ unsigned long long fx_stat(double e) { return (unsigned long long)llrint(e * kFxStat); }

template <typename R>
__global__ void __launch_bounds__(256, 3) transport_kernel(const RunParams P) {
    constexpr bool MX = sizeof(R) == 4;
    extern __shared__ unsigned char smem_raw[];
    __shared__ unsigned long long s_stats[kStCount];
    R* cache = reinterpret_cast<R*>(smem_raw);
    const int stride = blockDim.x;
    const int M = P.T.n_materials;
    R* thr = cache + threadIdx.x;
    R* mucache = cache + M * stride + threadIdx.x;
    if (threadIdx.x < kStCount) s_stats[threadIdx.x] = 0;
    __syncthreads();

    const V3<R> dom = {R(P.G.domain[0]), R(P.G.domain[1]), R(P.G.domain[2])};
    const V3<R> org = {R(P.G.origin[0]), R(P.G.origin[1]), R(P.G.origin[2])};
    const V3<R> ext = {R(P.G.ext[0]), R(P.G.ext[1]), R(P.G.ext[2])};
    const V3<R> spc = {R(P.G.spacing[0]), R(P.G.spacing[1]), R(P.G.spacing[2])};
    // the FP32 form multiplies by reciprocals (voxel index, free path); the FP64 form divides
    // exactly as the reference does
    const V3<R> ispc = {R(1) / spc.x, R(1) / spc.y, R(1) / spc.z};
    const int nx = P.G.dims[0], ny = P.G.dims[1], nz = P.G.dims[2];
    const bool have_tallies = P.n_tallies > 0;
    const uint64_t total_threads = uint64_t(gridDim.x) * blockDim.x;

    uint64_t h = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;  // current / next history id
    bool alive = false, pending = false;
    HistoryRng rng;
    V3<R> pos, dir, p0;
    R E = R(0), mu_max = R(0), inv_mu_max = R(0), s = R(0);
    int n_coh = 0, n_incoh = 0, vox = -1, mat = 0;
    uint32_t steps = 0, fetches = 0, trials = 0, words = 0;
    double hist_dep = 0.0;
    unsigned mask = 0xffffffffu;

    auto end_history = [&]() {
        if (P.trace) P.trace[h] = hist_dep;
        stat_add(s_stats, kStSteps, steps);
        stat_add(s_stats, kStFetches, fetches);
        stat_add(s_stats, kStTrials, trials);
        stat_add(s_stats, kStWords, words);
        alive = false;
        pending = false;
        h += total_threads;
    };

    for (;;) {
        const bool done = !alive && h >= P.n;
        mask = __ballot_sync(mask, !done);
        if (done) break;
        bool finish = false;  // the history ends in this iteration
        if (alive && !pending) {
            // one Woodcock step: getFreePath, move, domain test, voxel fetch, isDeltaScatter
            if (steps >= uint32_t(P.max_steps)) {
                stat_add(s_stats, kStStepCap, 1);
                finish = true;
            } else {
                ++steps;
                uint64_t w1, w2;
                rng.next_pair64(w1, w2);
                if constexpr (MX)
                    s = -log_(to_uniform(w1, R(0))) * inv_mu_max;
                else
                    s = -log_(to_uniform(w1, R(0))) / mu_max;
                p0 = pos;
                pos = {pos.x + s * dir.x, pos.y + s * dir.y, pos.z + s * dir.z};
                if (!(pos.x >= R(0) && pos.x <= dom.x && pos.y >= R(0) && pos.y <= dom.y && pos.z >= R(0) &&
                      pos.z <= dom.z)) {
                    if (have_tallies)
                        score_tallies<R, MX>(P, p0, dir, s, E, scatter_class(n_coh, n_incoh), 0, false, R(0), words);
                    stat_add(s_stats, kStEscE, fx_stat(double(E)));
                    finish = true;
                } else {
                    const V3<R> q = {pos.x - org.x, pos.y - org.y, pos.z - org.z};
                    vox = -1;
                    mat = P.G.background;
                    if (q.x >= R(0) && q.x <= ext.x && q.y >= R(0) && q.y <= ext.y && q.z >= R(0) && q.z <= ext.z) {
                        int ix, iy, iz;
                        if constexpr (MX) {
                            ix = int(q.x * ispc.x);
                            iy = int(q.y * ispc.y);
                            iz = int(q.z * ispc.z);
                        } else {
                            ix = int(q.x / spc.x);
                            iy = int(q.y / spc.y);
                            iz = int(q.z / spc.z);
                        }
                        if (ix >= nx || iy >= ny || iz >= nz) {
                            stat_add(s_stats, kStEdge, 1);  // the reference's vector::at would throw here
                            ix = min(ix, nx - 1);
                            iy = min(iy, ny - 1);
                            iz = min(iz, nz - 1);
                        }
                        vox = ix + iy * nx + iz * nx * ny;
                        mat = __ldg(P.G.ids + vox);
                        ++fetches;
                    }
                    if (to_uniform(w2, R(0)) < thr[mat * stride]) {
                        if (have_tallies)
                            score_tallies<R, MX>(P, p0, dir, s, E, scatter_class(n_coh, n_incoh), 0, false, R(0),
                                                 words);
                    } else {
                        pending = true;  // a real collision: an event
                    }
                }
            }
        }
        if (finish) end_history();
        // events: run the parked collisions and history starts once enough lanes wait
        const bool want = pending || (!alive && h < P.n);
        const unsigned wmask = __ballot_sync(mask, want);
        const unsigned fmask = __ballot_sync(mask, alive && !pending);
        if (want && (__popc(wmask) >= P.regroup || fmask == 0u)) {
            finish = false;
            if (!alive) {
                // PhotonSource::generatePhoton + a fresh per-history stream
                rng.init(P.seed, P.first + h);
                sample_source<R>(P.S, rng, pos, dir, E);
                stat_add(s_stats, kStHistories, 1);
                stat_add(s_stats, kStSourceE, fx_stat(double(E)));
                n_coh = n_incoh = 0;
                steps = fetches = trials = words = 0;
                hist_dep = 0.0;
                mu_max = refresh_energy<R>(P, E, thr, mucache, stride);
                inv_mu_max = R(1) / mu_max;
                alive = true;
            } else {
                pending = false;
                // setInteractionType (physics_engine.cpp:82-109)
                const DevMaterial& Mt = P.T.mat[mat];
                const R mu_tot = mucache[mat * stride];
                const R p_coh = spline_lookup<R>(P.T, Mt.coh, E) / mu_tot;
                const R p_incoh = spline_lookup<R>(P.T, Mt.incoh, E) / mu_tot;
                const R u3 = uniform<R>(rng);
                const int cls0 = scatter_class(n_coh, n_incoh);
                const R E0 = E;
                const V3<R> d0 = dir;
                R dep = R(0);
                bool energy_changed = false, failed = false;
                if (u3 < p_coh) {
                    // CoherentScattering::interact
                    ++n_coh;
                    stat_add(s_stats, kStCoh, 1);
                    R mu;
                    if (!rita_sample<R>(P.T, Mt.rita, E, uniform<R>(rng), mu)) {
                        stat_add(s_stats, kStRangeErr, 1);
                        failed = true;
                    } else {
                        R theta = acos_(mu);
                        R phi = R(2 * kPi) * uniform<R>(rng);
                        dir = rotate_direction(dir, theta, phi);
                    }
                } else if (u3 < p_coh + p_incoh) {
                    // IncoherentScattering::interact
                    ++n_incoh;
                    stat_add(s_stats, kStIncoh, 1);
                    R mu = R(1), kp = E / R(kMec2);
                    if (!sample_compton<R>(P, Mt, rng, E, mu, kp, trials)) {
                        stat_add(s_stats, kStTrialCap, 1);
                        failed = true;
                    } else {
                        const R k = E / R(kMec2);
                        R theta = acos_(mu);
                        R phi = R(2 * kPi) * uniform<R>(rng);
                        dir = rotate_direction(dir, theta, phi);
                        E = kp * R(kMec2);
                        dep = R(kMec2) * (k - kp);
                        energy_changed = true;
                    }
                } else {
                    // PhotoelectricEffect::interact
                    stat_add(s_stats, kStPhoto, 1);
                    dep = E;
                    finish = true;
                }
                if (failed) {
                    finish = true;
                } else {
                    if (have_tallies)
                        score_tallies<R, MX>(P, p0, d0, s, E0, cls0, scatter_class(n_coh, n_incoh), true, dep, words);
                    if (dep != R(0)) {
                        if (vox >= 0) {
                            stat_add(s_stats, kStDepGrid, fx_stat(double(dep)));
                            hist_dep += double(dep);
                            if (P.dose_stride) {
                                score_dose<MX>(P, vox, double(dep));
                                ++words;
                            }
                        } else {
                            stat_add(s_stats, kStDepBg, fx_stat(double(dep)));
                        }
                    }
                    if (!finish) {
                        if (!(fabs_(dir.x) <= R(2) && fabs_(dir.y) <= R(2) && fabs_(dir.z) <= R(2))) {
                            // a NaN direction (RITA rows below ~400 eV are NaN, as in the
                            // reference); its next step would leave the domain: retire the history
                            stat_add(s_stats, kStNonFinite, 1);
                            stat_add(s_stats, kStEscE, fx_stat(double(E)));
                            finish = true;
                        } else if (energy_changed) {
                            mu_max = refresh_energy<R>(P, E, thr, mucache, stride);
                            inv_mu_max = R(1) / mu_max;
                        }
                    }
                }
            }
            if (finish) end_history();
        }
    }
    __syncthreads();
    if (threadIdx.x < kStCount && s_stats[threadIdx.x]) atomicAdd(P.stats + threadIdx.x, s_stats[threadIdx.x]);
}
