// kernel_pool.cuh - the transport kernel with a per-warp photon pool (included by transport.cu
// after kernel_body.cuh, whose device functions it shares).
//
// Each warp owns kPoolSlots photon slots in shared memory, two per lane: the state a photon
// carries between events (position, direction, energy, Philox position, scatter counts,
// history counters) and its per-energy cache (majorant, every material's total cross section
// and delta threshold).  Each lane steps one photon - the Woodcock step of
// src/MIDSX/Core/physics_engine.cpp:28-79.  A photon that needs an event (a real collision, or
// a new history after its end) is parked in the warp's event list and the lane takes a photon
// from the warp's ready list at once, so the warp keeps stepping with all its lanes while
// events accumulate.  Once `regroup` events wait - or nothing is left to step - the warp runs
// up to 32 of them together, one per lane, and returns the surviving photons and the new
// histories to the ready list.
//
// Scheduling does not enter the physics: each history draws from its own Philox stream in the
// same order as in the lane-parking kernel, so the two kernels give the same trajectories, and
// bit-identical integer tallies in the mixed form.  Everything is warp-synchronous: a warp
// never waits for another warp, and the loop ends when the warp's lanes, ready list and event
// list are all empty after the launch's histories are handed out.

constexpr int kPoolSlots = 64;        // photon slots per warp
// Woodcock steps a lane takes per pass of the warp loop before the pool's bookkeeping
// (ready and event lists, ballots) runs.  Single-job kernels fix it at compile time (a
// run-time bound cost the cone-beam dose workload 1 %): 2 for the FP32 form with reference
// tracking, else 1 (default_steps_per_pass in transport.cu gives the measurements); batched
// kernels take RunParams::steps_per_pass (2 by default for the mixed form with reference
// tracking, the request server's launches included; the autotuner tries 1 and 2).  A photon
// that parks ends its pass early.
template <typename R, int TRACK>
__host__ __device__ constexpr int single_job_steps_per_pass() {
    return TRACK == MIDSX_TRACK_REFERENCE && sizeof(R) == 4 ? 2 : 1;
}
// A pass repeats, without the pool's list bookkeeping in between (the ready-list pickup,
// parking, and their ballots: a quarter of the warp cycles at one pass per round), while fewer
// than kPassWaitLanes lanes of the warp wait for a photon or an event, up to pass_repeats
// times.  Most Woodcock steps of a phantom in air are delta steps in the air, where a photon
// rarely parks, so the bookkeeping runs once per up to 16 steps there; inside the phantom
// collisions end the repeats early.  Cone-beam dose workload, FP32: +3.3 % for 8 repeats of
// two steps and a threshold of 16 lanes (8 of 8 lanes: +2.4 %, 16 repeats: +2.7 %; a ballot
// after every single step instead of every pass: +1.6 %).  One ballot per repeat.
constexpr int kPassWaitLanes = 16;
template <typename R, int TRACK>
__host__ __device__ constexpr int single_job_pass_repeats() {
    return TRACK == MIDSX_TRACK_REFERENCE && sizeof(R) == 4 ? 8 : 1;
}
constexpr uint32_t kKindFlight = 0u;  // slot kinds (meta bits 30-31)
constexpr uint32_t kKindCollide = 1u;
constexpr uint32_t kKindStart = 2u;

// meta word of a slot: job (bits 0-7), material (8-15), coherent (16-21) and incoherent
// (23-29) scatter counts saturated at 63 and 127 (only 0, 1 and "more" matter:
// scatter_class), the flight segment's step parity (22: HistoryRng), kind (30-31).
__device__ __forceinline__ uint32_t pack_meta(int job, int mat, int n_coh, int n_incoh, uint32_t kind,
                                              uint32_t par = 0u) {
    return uint32_t(job) | (uint32_t(mat) << 8) | (uint32_t(min(n_coh, 63)) << 16) | (par << 22) |
           (uint32_t(min(n_incoh, 127)) << 23) | (kind << 30);
}

// Shared-memory arrays over the block's slots (structure of arrays: lanes touch consecutive
// words when they hold consecutive slots).
template <typename R>
struct PoolSlots {
    R *px, *py, *pz, *dx, *dy, *dz, *e, *mumax, *qx, *qy, *qz, *s;  // q = start of the last step
    uint32_t *rn, *h0, *h1, *steps, *fetches, *words, *vox, *meta;
    R *thr, *mu;  // per-energy cache, [material][slot]
};

constexpr int kPoolRealWords = 12;  // R arrays per slot
constexpr int kPoolIntWords = 8;    // uint32 arrays per slot

// Batched launches (MULTI) run job-affine blocks: a block works on one job at a time and holds
// only that job in shared memory - its record (DevJob), its geometry in the working
// precision, its run statistics and the block's control words - about 1 KB.  Blocks start
// spread over the jobs in proportion to their histories; a block whose job has no histories
// left to hand out lets its warps finish their photons (drain), flushes the job's statistics
// and moves to the job with the most histories left.  Steps and events then run as in a
// single-job launch, 7 blocks of 128 threads per SM (every job's counters and geometry in
// shared memory, ~16 KB for 64 jobs, held batched launches to 24 warps per SM), and the tails of
// different jobs overlap.  Each job hands out its histories from a counter of its own.
constexpr int kBlockCtlWords = 4;  // current job, its histories this launch, spare
constexpr int kBlockKeyWords = 20;  // the job's Philox key schedule (philox_round_keys)
template <typename R>
__host__ __device__ inline size_t pool_head_bytes(int n_jobs, bool multi) {
    (void)n_jobs;
    size_t b = size_t(kStCount) * 8;
    if (multi)
        b += sizeof(DevJob) + ((sizeof(Geo<R>) + 15) & ~size_t(15)) + kBlockCtlWords * 8 + kBlockKeyWords * 4;
    return (b + 15) & ~size_t(15);
}

// The job a block works on: its record in shared memory (batched) or the launch's own job0.
template <bool MULTI>
__device__ __forceinline__ const DevJob& pick_job(const RunParams& P, const DevJob* s_job) {
    if constexpr (MULTI)
        return *s_job;
    else
        return P.job0;
}
template <bool MULTI, typename R>
__device__ __forceinline__ const Geo<R>& pick_geo(const RunParams& P, const Geo<R>* s_geo) {
    if constexpr (MULTI)
        return *s_geo;
    else
        return job0_geo(P, R(0));
}

// Batched launches: the next job of a block (warp 0 decides, all lanes return it): the job
// whose history range holds the block's share of the launch on its first call, else the job
// with the most histories left to hand out; -1 when every job is handed out.
__device__ __forceinline__ int next_block_job(const RunParams& P, bool first) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long total = P.prefix[P.n_jobs];
    if (first) {
        const unsigned long long target =
            (unsigned long long)((double(blockIdx.x) + 0.5) * double(total) / double(gridDim.x));
        int lo = 0, hi = P.n_jobs;  // last job with prefix <= target
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (P.prefix[mid] <= target) lo = mid;
            else hi = mid;
        }
        const unsigned long long n = P.prefix[lo + 1] - P.prefix[lo];
        const unsigned long long c = *reinterpret_cast<volatile const unsigned long long*>(P.job_counters + lo);
        if (c < n) return lo;
    }
    unsigned long long best = 0;
    int best_j = -1;
    for (int j = int(lane); j < P.n_jobs; j += 32) {
        const unsigned long long n = P.prefix[j + 1] - P.prefix[j];
        const unsigned long long c = *reinterpret_cast<volatile const unsigned long long*>(P.job_counters + j);
        const unsigned long long rem = c < n ? n - c : 0ull;
        if (rem > best) {
            best = rem;
            best_j = j;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oj = __shfl_xor_sync(0xffffffffu, best_j, o);
        if (ob > best || (ob == best && oj >= 0 && (best_j < 0 || oj < best_j))) {
            best = ob;
            best_j = oj;
        }
    }
    return best_j;
}

// Shared-memory bytes of a pool launch: per-job counters, batch prefix and geometry, the
// slots, each warp's 32-word scratch for aggregated tallies, then each warp's ready and
// event lists (one byte per entry).
template <typename R>
__host__ __device__ inline size_t pool_scratch_offset(int n_jobs, bool multi, int n_materials, int block) {
    const size_t ns = size_t(block / 32) * kPoolSlots;
    size_t b = pool_head_bytes<R>(n_jobs, multi);
    b += ns * (kPoolRealWords * sizeof(R) + kPoolIntWords * 4 + 2 * size_t(n_materials) * sizeof(R));
    return (b + 15) & ~size_t(15);
}

template <typename R>
__host__ __device__ inline size_t pool_smem(int n_jobs, bool multi, int n_materials, int block) {
    return pool_scratch_offset<R>(n_jobs, multi, n_materials, block) + size_t(block / 32) * 32 * 8 +
           size_t(block / 32) * 2 * kPoolSlots;
}

// TRACK = midsx_tracking, each a kernel of its own (compiled into one kernel with the
// reference tracking, the background fast path's code cost the reference path 8 %).  SPEC:
// the launch keeps incident-energy spectra (a kernel of its own too: the spectrum code cost
// tally-free launches 5 %).  Batched
// launches hold one job per block (job-affine blocks, above).  FP32 launches run 7 blocks of
// 128 threads per SM (72 registers, a few bytes spilled): +6.5 % against 6 blocks of 80
// registers on the cone-beam dose workload.
template <typename R, bool MULTI, int TRACK, bool SPEC = false>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 7 : 4) transport_pool_kernel(const RunParams P) {
    constexpr bool MX = sizeof(R) == 4;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int njobs = 1;  // the statistics in shared memory are those of the block's one job
    const int M = P.T.n_materials;
    unsigned long long* s_stats = reinterpret_cast<unsigned long long*>(smem_raw);
    // batched: the block's job record, its geometry and the block's control words
    DevJob* s_job = reinterpret_cast<DevJob*>(s_stats + kStCount);
    Geo<R>* s_geo = reinterpret_cast<Geo<R>*>(reinterpret_cast<unsigned char*>(s_job) + sizeof(DevJob));
    long long* s_ctl = reinterpret_cast<long long*>(reinterpret_cast<unsigned char*>(s_geo) +
                                                    ((sizeof(Geo<R>) + 15) & ~size_t(15)));
    uint32_t(&s_rk)[kBlockKeyWords] = *reinterpret_cast<uint32_t(*)[kBlockKeyWords]>(s_ctl + kBlockCtlWords);
    const int nw = int(blockDim.x >> 5);
    const int ns = nw * kPoolSlots;
    PoolSlots<R> S;
    {
        unsigned char* p = smem_raw + pool_head_bytes<R>(njobs, MULTI);
        R** reals[kPoolRealWords] = {&S.px, &S.py, &S.pz, &S.dx, &S.dy, &S.dz, &S.e, &S.mumax,
                                     &S.qx, &S.qy, &S.qz, &S.s};
        for (int i = 0; i < kPoolRealWords; ++i) {
            *reals[i] = reinterpret_cast<R*>(p);
            p += size_t(ns) * sizeof(R);
        }
        S.thr = reinterpret_cast<R*>(p);
        p += size_t(ns) * M * sizeof(R);
        S.mu = reinterpret_cast<R*>(p);
        p += size_t(ns) * M * sizeof(R);
        uint32_t** ints[kPoolIntWords] = {&S.rn, &S.h0, &S.h1, &S.steps, &S.fetches, &S.words, &S.vox, &S.meta};
        for (int i = 0; i < kPoolIntWords; ++i) {
            *ints[i] = reinterpret_cast<uint32_t*>(p);
            p += size_t(ns) * 4;
        }
    }
    uint8_t* stacks = smem_raw + pool_smem<R>(njobs, MULTI, M, int(blockDim.x)) - size_t(nw) * 2 * kPoolSlots;
    unsigned long long* scratch = reinterpret_cast<unsigned long long*>(
                                      smem_raw + pool_scratch_offset<R>(njobs, MULTI, M, int(blockDim.x))) +
                                  (threadIdx.x >> 5) * 32;
    if constexpr (!MULTI)
        for (int i = threadIdx.x; i < kStCount; i += blockDim.x) s_stats[i] = 0;
    const unsigned lane = threadIdx.x & 31u;
    const int warp = int(threadIdx.x >> 5);
    const unsigned below = (1u << lane) - 1u;
    const int sbase = warp * kPoolSlots;
    uint8_t* rdy = stacks + warp * 2 * kPoolSlots;  // ready list: slots to step
    uint8_t* evq = rdy + kPoolSlots;               // event list: slots waiting for an event
    // every slot starts as a history start (a batched block again for each of its jobs)
    auto init_pool = [&]() {
        evq[lane] = uint8_t(lane);
        evq[lane + 32] = uint8_t(lane + 32);
        S.meta[sbase + lane] = pack_meta(0, 0, 0, 0, kKindStart);
        S.meta[sbase + lane + 32] = pack_meta(0, 0, 0, 0, kKindStart);
    };
    if constexpr (!MULTI) {
        init_pool();
        __syncthreads();
    }
    const Geo<R>& g0 = pick_geo<MULTI, R>(P, s_geo);
    const DevJob& J = pick_job<MULTI>(P, s_job);
    const unsigned long long epoch = P.epoch ? *P.epoch : 0ull;
    const int regroup = max(1, min(P.regroup, 32));
    constexpr bool fast_mode = TRACK != MIDSX_TRACK_REFERENCE;   // background flights
    constexpr bool macro_mode = TRACK == MIDSX_TRACK_MACRO_CELL;  // and macro-cell flights in grids
    int rdy_top = 0, ev_top = kPoolSlots;  // warp-uniform list sizes
    bool exhausted = false;                // warp-uniform: every history of the job handed out
    // batched: the block's job's history counter and its histories in this launch (a single
    // job reads the launch's own from the kernel parameters)
    unsigned long long* job_counter = nullptr;
    unsigned long long job_total = 0;

    // the photon in this lane's registers
    int cur = -1;  // slot stepped by this lane
    V3<R> pos, dir, p0;
    R E = R(0), mu_max = R(1), inv_mu_max = R(1), s = R(0);
    HistoryRng rng;
    int job = 0, mat = 0, vox = -1, n_coh = 0, n_incoh = 0, ntal = 0;
    uint32_t kind = kKindFlight, steps = 0, fetches = 0, trials = 0, words = 0;
    uint32_t spar = 0u;  // step parity at the start of the flight segment (HistoryRng)
    uint32_t sw2 = 0u, sw3 = 0u;  // the step block's second word pair, for the pass's next step

    // Slot traffic is kept to the fields each transition needs.  In flight a photon changes
    // only its position, Philox position and counters; the collision site (step start, length,
    // voxel, material) matters only to the event that follows.
    auto load_flight = [&](int sl) {  // what a step needs
        pos = {S.px[sl], S.py[sl], S.pz[sl]};
        dir = {S.dx[sl], S.dy[sl], S.dz[sl]};
        E = S.e[sl];
        mu_max = S.mumax[sl];
        inv_mu_max = R(1) / mu_max;
        const uint32_t meta = S.meta[sl];
        job = int(meta & 0xffu);
        n_coh = int((meta >> 16) & 0x3fu);
        spar = (meta >> 22) & 1u;
        n_incoh = int((meta >> 23) & 0x7fu);
        kind = meta >> 30;
        const uint64_t seed = J.seed;
        rng.k0 = uint32_t(seed);
        rng.k1 = uint32_t(seed >> 32);
        rng.h0 = S.h0[sl];
        rng.h1 = S.h1[sl];
        rng.n = S.rn[sl];
        // the unused words of an event block are never drawn after the event: the next
        // interaction starts a new block (HistoryRng::align_event)
        rng.b1 = rng.b2 = rng.b3 = 0u;
        steps = S.steps[sl];
        fetches = S.fetches[sl];
        words = S.words[sl];
        // fast tracking steers by the last lookup's region (-1: background, -2: not known)
        if constexpr (fast_mode) vox = int(S.vox[sl]);
        ntal = J.n_tallies;
    };
    auto load_event = [&](int sl) {  // a parked photon: flight state plus its collision site
        load_flight(sl);
        p0 = {S.qx[sl], S.qy[sl], S.qz[sl]};
        s = S.s[sl];
        mat = int((S.meta[sl] >> 8) & 0xffu);
        vox = int(S.vox[sl]);
    };
    auto save_flight = [&](int sl) {  // what a step changes
        S.px[sl] = pos.x;
        S.py[sl] = pos.y;
        S.pz[sl] = pos.z;
        S.rn[sl] = rng.n;
        S.steps[sl] = steps;
        S.fetches[sl] = fetches;
        S.words[sl] = words;
        if constexpr (fast_mode) S.vox[sl] = uint32_t(vox);
    };
    auto save_collision = [&](int sl) {  // a photon parked at a real collision
        save_flight(sl);
        S.qx[sl] = p0.x;
        S.qy[sl] = p0.y;
        S.qz[sl] = p0.z;
        S.s[sl] = s;
        S.vox[sl] = uint32_t(vox);
        S.meta[sl] = pack_meta(job, mat, n_coh, n_incoh, kKindCollide, spar);
    };
    auto save_after_event = [&](int sl) {  // a photon leaving an event (or a new history)
        save_flight(sl);
        S.dx[sl] = dir.x;
        S.dy[sl] = dir.y;
        S.dz[sl] = dir.z;
        S.e[sl] = E;
        S.mumax[sl] = mu_max;
        S.h0[sl] = rng.h0;
        S.h1[sl] = rng.h1;
        S.meta[sl] = pack_meta(job, mat, n_coh, n_incoh, kKindFlight, spar);
    };
    // Compton trials go to the statistics at the event itself (sample_compton counts them)
    auto end_history = [&]() {
        unsigned long long* st = s_stats + job * kStCount;
        stat_add(st, kStSteps, steps);
        stat_add(st, kStFetches, fetches);
        stat_add(st, kStWords, words);
    };

    // single job: one pass of the job loop; batched: one per job the block works on
    bool first_job = true;
    do {
    if constexpr (MULTI) {
        if (warp == 0) {
            const int j = next_block_job(P, first_job);
            if (lane == 0) {
                s_ctl[0] = j;
                s_ctl[1] = j >= 0 ? (long long)(P.prefix[j + 1] - P.prefix[j]) : 0;
            }
        }
        __syncthreads();
        const int j = int(s_ctl[0]);
        if (j < 0) break;
        // the job's record to shared memory, its geometry in the working precision
        {
            const unsigned* src = reinterpret_cast<const unsigned*>(P.jobs + j);
            unsigned* dst = reinterpret_cast<unsigned*>(s_job);
            for (int i = threadIdx.x; i < int(sizeof(DevJob) / 4); i += blockDim.x) dst[i] = src[i];
        }
        if (threadIdx.x == 0) {
            *s_geo = make_geo<R>(P.jobs[j].G);
            philox_round_keys(P.jobs[j].seed, s_rk);
        }
        job_counter = P.job_counters + j;
        job_total = (unsigned long long)s_ctl[1];
        for (int i = threadIdx.x; i < kStCount; i += blockDim.x) s_stats[i] = 0;
        init_pool();
        rdy_top = 0;
        ev_top = kPoolSlots;
        exhausted = false;
        cur = -1;
        __syncthreads();
    }
    for (;;) {
        // lanes without a photon take one from the ready list
        {
            const bool want = cur < 0;
            const unsigned wm = __ballot_sync(FULL, want);
            const int r = __popc(wm & below);
            if (want && r < rdy_top) {
                cur = sbase + rdy[rdy_top - 1 - r];
                load_flight(cur);
            }
            rdy_top -= min(__popc(wm), rdy_top);
        }
        if (__ballot_sync(FULL, cur >= 0) == 0u && rdy_top == 0 && ev_top == 0) break;
        uint32_t park = kKindFlight;
        const int npass = MULTI ? P.steps_per_pass : single_job_steps_per_pass<R, TRACK>();
        const int repeats = MULTI ? P.pass_repeats : single_job_pass_repeats<R, TRACK>();
        for (int rep = 0; rep < repeats; ++rep) {
        if (rep > 0 && __popc(__ballot_sync(FULL, cur < 0 || park != kKindFlight)) >= kPassWaitLanes) break;
        for (int pass = 0; pass < npass && park == kKindFlight && cur >= 0; ++pass) {
            bool segment = false;  // the step's segment goes to the tallies (escape or delta step)
            if (cur >= 0) {
                // one Woodcock step: getFreePath, move, domain test, voxel fetch, isDeltaScatter
                const Geo<R>& g = g0;
                unsigned long long* st = s_stats + job * kStCount;
                if (steps >= uint32_t(P.max_steps)) {
                    stat_add(st, kStStepCap, 1);
                    park = kKindStart;
                } else {
                    // the step's uniforms: the word pair (0, 1) of its block for an even step
                    // index, (2, 3) for an odd one.  A flight segment starts even and passes
                    // run two steps, so a pass computes one block and its second step takes
                    // the pair kept from the first; a step of odd index in a pass's first
                    // step (one step per pass, or a segment start in mid-pass) recomputes.
                    const uint32_t si = steps + spar;
                    ++steps;
                    uint32_t wa, wb;
                    if (pass == 0 || !(si & 1u)) {
                        Philox4 q;
                        if constexpr (MULTI)
                            q = rng.step_block_rk(si, s_rk);
                        else
                            q = rng.step_block_rk(si, P.round_keys);
                        wa = (si & 1u) ? q.v[2] : q.v[0];
                        wb = (si & 1u) ? q.v[3] : q.v[1];
                        sw2 = q.v[2];
                        sw3 = q.v[3];
                    } else {
                        wa = sw2;
                        wb = sw3;
                    }
                    const uint64_t w1 = uint64_t(wa) << 32, w2 = uint64_t(wb) << 32;
                    // MIDSX_TRACK_BACKGROUND_FAST: a photon known to be in the background (vox == -1
                    // after its last voxel lookup) flies against the background's own attenuation,
                    // exact there, up to the first grid it would enter
                    // MIDSX_TRACK_MACRO_CELL: any other photon spends one optical depth through the
                    // macro cells of the grid it is in.  fl: -1 a reference step; 0 a tentative
                    // collision against the cell majorant mu_c; 1 a flight that ends, without
                    // interaction, kCutSliver past a face; 2 a tentative collision in that sliver
                    // (against the global majorant); 3 a background collision (always real)
                    int fl = -1;
                    R mu_c = R(0);
                    if (fast_mode) {
                        R tau, tau_rem = R(0), lim = R(INFINITY);
                        if constexpr (MX)
                            tau = fmaxf(-__logf(to_uniform(w1, R(0))), 0.0f);
                        else
                            tau = -log_(to_uniform(w1, R(0)));
                        bool bg = vox == -1;
                        if (macro_mode && !bg) {
                            fl = cell_flight<R, MX>(g, J.G, S.mu + cur, ns, pos, dir, tau,
                                                    s, mu_c, tau_rem);
                            bg = fl == 2;
                        }
                        if (bg) {
                            const R mu_bg = S.mu[g.bg * ns + cur];
                            s = tau / mu_bg;
                            lim = grid_entry<R, MX>(g, pos, dir);
                            fl = 3;
                            if (s > lim) {
                                tau_rem = tau - mu_bg * lim;
                                s = lim;
                                fl = 1;
                            }
                        }
                        if (fl == 1) {
                            const R past = tau_rem * inv_mu_max;
                            if (past < R(kCutSliver)) {
                                s += past;
                                fl = 2;
                            } else {
                                s += R(kCutSliver);
                            }
                        }
                    }
                    if (fl >= 0) {
                        // s from the flight above
                    } else if constexpr (MX) {
                        s = fmaxf(-__logf(to_uniform(w1, R(0))), 0.0f) * inv_mu_max;
                    } else {
                        s = -log_(to_uniform(w1, R(0))) * inv_mu_max;
                    }
                    p0 = pos;
                    pos = {pos.x + s * dir.x, pos.y + s * dir.y, pos.z + s * dir.z};
                    if (!(pos.x >= R(0) && pos.x <= g.dom.x && pos.y >= R(0) && pos.y <= g.dom.y && pos.z >= R(0) &&
                          pos.z <= g.dom.z)) {
                        stat_add(st, kStEscE, fx_stat(E));
                        segment = true;
                        park = kKindStart;
                    } else if (fl == 3) {
                        mat = g.bg;
                        vox = -1;
                        park = kKindCollide;  // every background collision is real
                    } else if (fl == 1) {
                        // past a face, no interaction: the next flight finds its region from here
                        // (BACKGROUND_FAST: a reference step, valid everywhere)
                        vox = -2;
                        segment = true;
                    } else if (fl == 0) {
                        // real with probability mu(voxel) / mu(cell); a voxel met across a cell face
                        // by rounding, with a larger attenuation than the cell's, interacts
                        locate<R, MX>(g, pos, vox, mat, fetches, st);
                        const R mm = S.mu[mat * ns + cur];
                        if (to_uniform(w2, R(0)) * mu_c < mu_c - mm)
                            segment = true;
                        else
                            park = kKindCollide;
                    } else {
                        locate<R, MX>(g, pos, vox, mat, fetches, st);
                        if (to_uniform(w2, R(0)) < S.thr[mat * ns + cur])
                            segment = true;
                        else
                            park = kKindCollide;  // a real collision
                    }
                }
            }
            // surface and volume tallies see every step that does not interact, the last (escaping)
            // one included (physics_engine.cpp:48-49).  Scored per lane: nearly every step runs
            // this and almost none touches a tally, so the warp-collective form (used for the
            // collisions below) measured 3 % slower on the cone-beam dose workload and 29 % slower
            // on the radiography workload.
            if (segment && ntal > 0)
                score_tallies<R, MX, SPEC>(J.tallies, ntal, p0, dir, s, E,
                                     scatter_class(n_coh, n_incoh), 0, false, R(0), words);
        }  // pass
        }  // repeats
        if (cur >= 0 && park == kKindStart) end_history();
        // photons that need an event go to the event list
        {
            const bool parks = park != kKindFlight;
            const unsigned pm = __ballot_sync(FULL, parks);
            if (parks) {
                if (park == kKindCollide)
                    save_collision(cur);
                else
                    S.meta[cur] = pack_meta(0, 0, 0, 0, kKindStart);
                evq[ev_top + __popc(pm & below)] = uint8_t(cur - sbase);
                cur = -1;
            }
            ev_top += __popc(pm);
        }
        __syncwarp();
        const bool idle = __ballot_sync(FULL, cur >= 0) == 0u;
        if (!(ev_top >= regroup || (idle && rdy_top == 0 && ev_top > 0))) continue;

        // ------------------------------------------------------------ event phase ---
        if (cur >= 0) save_flight(cur);  // the stepping photons wait in their slots
        __syncwarp();
        const int n_ev = min(ev_top, 32);
        int sl = int(lane) < n_ev ? sbase + evq[ev_top - 1 - int(lane)] : -1;
        ev_top -= n_ev;
        bool need_start = false, need_refresh = false, scored = false, ended = false;
        R dep = R(0), E0 = R(0);
        V3<R> d0 = {R(0), R(0), R(0)};
        int cls0 = 0;
        if (sl >= 0) {
            load_event(sl);
            if (kind != kKindCollide) {
                need_start = true;
            } else {
                unsigned long long* st = s_stats + job * kStCount;
                bool finish = false;
                // setInteractionType (physics_engine.cpp:82-109)
                const DevMaterial& Mt = P.T.mat[mat];
                const R mu_tot = S.mu[mat * ns + sl];
                R p_coh, p_incoh;
                interaction_probs<R>(P.T, Mt, E, mu_tot, p_coh, p_incoh);
                rng.align_event();
                const R u3 = uniform<R>(rng);
                cls0 = scatter_class(n_coh, n_incoh);
                E0 = E;
                d0 = dir;
                R mu_s = R(1);
                bool energy_changed = false, failed = false, scattered = false;
                if (u3 < p_coh) {
                    // CoherentScattering::interact
                    ++n_coh;
                    stat_add(st, kStCoh, 1);
                    R mu;
                    if (!rita_sample<R>(P.T, Mt.rita, E, uniform<R>(rng), mu)) {
                        stat_add(st, kStRangeErr, 1);
                        failed = true;
                    } else {
                        mu_s = mu;
                        scattered = true;
                    }
                } else if (u3 < p_coh + p_incoh) {
                    // IncoherentScattering::interact
                    ++n_incoh;
                    stat_add(st, kStIncoh, 1);
                    R mu = R(1), kp = E / R(kMec2);
                    trials = 0;
                    const bool sampled = sample_compton<R>(P, Mt, rng, E, mu, kp, trials);
                    stat_add(st, kStTrials, trials);
                    if (!sampled) {
                        stat_add(st, kStTrialCap, 1);
                        failed = true;
                    } else {
                        const R k = E / R(kMec2);
                        mu_s = mu;
                        scattered = true;
                        E = kp * R(kMec2);
                        dep = R(kMec2) * (k - kp);
                        energy_changed = true;
                    }
                } else {
                    // PhotoelectricEffect::interact
                    stat_add(st, kStPhoto, 1);
                    dep = E;
                    finish = true;
                }
                // both scatterings end with the new direction (azimuth drawn last, as in each
                // interaction's own order): one call serves the coherent and incoherent lanes
                if (scattered) dir = scatter_dir(dir, mu_s, uniform<R>(rng));
                if (failed) {
                    finish = true;
                } else {
                    scored = true;  // tallies and dose below, with the whole warp
                    if (dep != R(0)) stat_add(st, vox >= 0 ? kStDepGrid : kStDepBg, fx_stat(dep));
                    if (!finish) {
                        if (!(fabs_(dir.x) <= R(2) && fabs_(dir.y) <= R(2) && fabs_(dir.z) <= R(2))) {
                            // a NaN direction (RITA rows below ~400 eV are NaN, as in the
                            // reference); its next step would leave the domain: retire the history
                            stat_add(st, kStNonFinite, 1);
                            stat_add(st, kStEscE, fx_stat(E));
                            finish = true;
                        } else if (energy_changed) {
                            need_refresh = true;
                        }
                    }
                }
                spar = steps & 1u;  // a new flight segment (HistoryRng)
                ended = finish;
            }
        }
        // the collisions' tallies and voxel dose, aggregated over the warp
        if (__any_sync(FULL, scored && ntal > 0))
            score_tallies_warp<R, MX, SPEC>(scored && ntal > 0, J.tallies, ntal, p0, d0,
                                      s, E0, cls0, scatter_class(n_coh, n_incoh), true, dep, words, scratch);
        {
            const bool dosed = scored && dep != R(0) && vox >= 0 && J.dose_stride != 0;
            if (dosed) ++words;
            warp_record<R, MX>(dosed ? kRecDose : kRecNone, dosed ? J.dose + size_t(vox) * J.dose_stride : nullptr,
                               J.dose_stride, dep, R(0), scratch);
        }
        if (ended) {
            end_history();
            need_start = true;
        }
        // new histories: one atomic per warp hands out the lanes' history indices
        const unsigned nm = __ballot_sync(FULL, need_start);
        if (nm) {
            const unsigned long long total = MULTI ? job_total : P.total;
            unsigned long long base = total;
            if (!exhausted) {
                const int leader = __ffs(nm) - 1;
                if (int(lane) == leader)
                    base = atomicAdd(MULTI ? job_counter : P.counter, (unsigned long long)__popc(nm));
                base = __shfl_sync(FULL, base, leader);
                if (base + (unsigned long long)__popc(nm) >= total) exhausted = true;
            }
            if (need_start) {
                const unsigned long long gidx = base + (unsigned long long)__popc(nm & below);
                if (gidx >= total) {
                    sl = -1;  // nothing left to start: the slot stays empty
                } else {
                    job = 0;
                    const uint64_t hid = J.first + epoch * J.n + gidx;
                    ntal = J.n_tallies;
                    // PhotonSource::generatePhoton + a fresh per-history stream
                    rng.init(J.seed, hid);
                    sample_source<R>(J.S, rng, pos, dir, E);
                    unsigned long long* sj = s_stats + job * kStCount;
                    stat_add(sj, kStHistories, 1);
                    stat_add(sj, kStSourceE, fx_stat(E));
                    n_coh = n_incoh = 0;
                    steps = fetches = trials = words = 0;
                    spar = 0u;
                    mat = 0;
                    vox = -2;  // region of the source point not looked up yet
                    s = R(0);
                    p0 = pos;
                    need_refresh = true;
                }
            }
        }
        // per-energy cache of Compton survivors and new histories, in one call
        if (need_refresh) {
            if constexpr (MULTI || !MX)
                mu_max = refresh_energy<R>(P, E, S.thr + sl, S.mu + sl, ns);
            else
                mu_max = refresh_energy_call<R>(P, E, S.thr + sl, S.mu + sl, ns);
            inv_mu_max = R(1) / mu_max;
        }
        // survivors and new histories go to the ready list
        {
            const bool ready = sl >= 0;
            if (ready) save_after_event(sl);
            const unsigned rm = __ballot_sync(FULL, ready);
            if (ready) rdy[rdy_top + __popc(rm & below)] = uint8_t(sl - sbase);
            rdy_top += __popc(rm);
        }
        __syncwarp();
        if (cur >= 0) load_flight(cur);  // back to the photon this lane was stepping
    }
    // the job's histories are done in this block (the warps drained their pools)
    __syncthreads();
    for (int i = threadIdx.x; i < kStCount; i += blockDim.x) {
        const unsigned long long v = s_stats[i];
        if (v) atomicAdd(J.stats + i, v);
    }
    if constexpr (MULTI) __syncthreads();  // the record and statistics are read before the next job replaces them
    first_job = false;
    } while (MULTI);  // jobs
}
