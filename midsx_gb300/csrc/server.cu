// server.cu - request server with continuous batching on one GPU (midsx_server_* in
// include/midsx_gpu.h).  Host code only: the transport runs in the batched form of the
// kernel of transport.cu, reached through runtime.h.
//
// Threads.  Client threads submit, poll, wait, read and release; one scheduler thread owns
// every stream operation of the server (pool allocations and frees, uploads, job records,
// launches) and the retirement of finished launches.  One mutex guards the request table,
// the admission queue, the phantom table and the statistics.
//
// Device memory.  Phantom storage and request tallies come from one stream-ordered memory
// pool, allocated and freed on the setup stream, so that admissions and releases never wait
// for the kernels that run (cudaMalloc / cudaFree would).  The budget is enforced by the
// host-side count of charged bytes: tallies of every admitted and not yet released request
// plus every resident phantom.
//
// Launches.  Each launch slot has its own stream, pinned host records, device records,
// history offsets and history counter.  A slot is refilled as soon as its previous launch has
// completed; with two or more slots one launch is always queued behind the running one, so
// the GPU does not idle while the host forms the next launch, and the tail of one launch
// overlaps the start of the next.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/midsx_gpu.h"
#include "runtime.h"
#include "tables_internal.h"

namespace {

using Clock = std::chrono::steady_clock;
constexpr int kMaxJobs = MIDSX_MAX_BATCH_JOBS;
constexpr int kMaxSlots = 4;

struct Phantom {
    midsx_phantom_h h = nullptr;
    midsx_tables_h tables = nullptr;  // the cross-section tables its requests run with
    std::vector<uint8_t> host;  // dense (material-index) voxels, for uploads after an eviction
    size_t bytes = 0;
    uint8_t* dev = nullptr;     // pool storage; nullptr = not resident
    int refs = 0;               // admitted requests that use it
    uint64_t last_use = 0;
};

struct Request {
    uint64_t id = 0;
    midsx_request r{};
    std::vector<midsx_tally_spec> specs;
    int state = MIDSX_REQ_QUEUED;
    midsx_status status = MIDSX_OK;
    std::string error;
    midsx_tallies_h tallies = nullptr;
    size_t tally_bytes = 0;
    size_t footprint = 0;
    uint64_t scheduled = 0, done = 0;
    int launches = 0;
    int in_flight = 0;      // launches holding this request that have not completed
    bool released = false;  // the client is done with it; free once in_flight == 0
    bool pinned = false;    // holds a reference on its phantom (admitted, launches may read it)
    uint64_t admit_seq = 0;
    uint64_t last_launch = 0;  // number of the last launch that included it (0 = none yet)
    double t_submit = -1, t_admit = -1, t_first = -1, t_done = -1;
};

struct Part {
    Request* req;
    uint64_t n;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr, end = nullptr;
    unsigned char* host_jobs = nullptr;       // pinned, kMaxJobs records
    unsigned long long* host_prefix = nullptr;  // pinned, kMaxJobs + 1 offsets
    void* dev_jobs = nullptr;
    unsigned long long* dev_prefix = nullptr;
    unsigned long long* dev_counter = nullptr;
    bool busy = false;
    std::vector<Part> parts;
    Clock::time_point issued;
};

}  // namespace

struct midsx_gpu_server {
    midsx_tables_h tables = nullptr;  // default tables of registered phantoms
    int device = 0;
    midsx_server_config cfg{};
    uint64_t budget = 0;
    uint64_t launch_histories = 0;
    int max_active = kMaxJobs;
    int n_slots = 2;
    double deadline_s = 1800.0;

    cudaMemPool_t pool = nullptr;
    cudaStream_t setup = nullptr;
    cudaEvent_t setup_done = nullptr;  // recorded after each batch of setup work
    bool setup_recorded = false;
    Slot slots[kMaxSlots];

    std::mutex mu;
    std::condition_variable cv_sched;  // wakes the scheduler: submission, release, stop
    std::condition_variable cv_done;   // wakes waiters: a request finished or failed
    std::thread worker;
    bool stop = false;
    bool broken = false;  // a launch failed or timed out: the device state is unknown

    std::vector<std::unique_ptr<Phantom>> phantoms;
    std::map<uint64_t, std::unique_ptr<Request>> requests;
    std::deque<Request*> queue;    // submitted, not admitted (arrival order)
    std::vector<Request*> active;  // admitted, histories left to schedule or in flight
    std::vector<Request*> to_free; // released requests whose memory the scheduler returns
    uint64_t next_id = 1;
    uint64_t admit_counter = 0;
    uint64_t use_clock = 0;
    Clock::time_point t0;
    midsx_server_stats st{};

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    void run();
    bool retire_locked();
    bool admit_locked(bool& enqueued_setup);
    bool launch_locked();
    void fail_locked(Request* r, midsx_status s, const std::string& why);
    void unpin_locked(Request* r);
    void free_request_memory_locked(Request* r);
};

namespace {

bool ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    midsx::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

}  // namespace

void midsx_gpu_server::fail_locked(Request* r, midsx_status s, const std::string& why) {
    if (r->state == MIDSX_REQ_FAILED || r->state == MIDSX_REQ_DONE) return;
    const bool was_active = r->state == MIDSX_REQ_RUNNING;
    r->state = MIDSX_REQ_FAILED;
    r->status = s;
    r->error = why;
    r->t_done = now();
    st.failed++;
    if (was_active) active.erase(std::remove(active.begin(), active.end(), r), active.end());
    unpin_locked(r);
    cv_done.notify_all();
}

// A finished request lets go of its phantom once no launch that reads it is in flight.
void midsx_gpu_server::unpin_locked(Request* r) {
    if (!r->pinned || r->in_flight > 0 || (r->state != MIDSX_REQ_DONE && r->state != MIDSX_REQ_FAILED)) return;
    phantoms[size_t(r->r.phantom)]->refs--;
    r->pinned = false;
}

void midsx_gpu_server::free_request_memory_locked(Request* r) {
    if (r->tallies) {
        midsx::rt::tallies_destroy_async(r->tallies, setup);
        r->tallies = nullptr;
    }
}

// Completed launches: histories done, requests finished.  Returns true if anything changed.
bool midsx_gpu_server::retire_locked() {
    bool changed = false;
    for (int i = 0; i < n_slots; ++i) {
        Slot& s = slots[i];
        if (!s.busy) continue;
        cudaError_t q = cudaEventQuery(s.end);
        if (q == cudaErrorNotReady) {
            if (std::chrono::duration<double>(Clock::now() - s.issued).count() > deadline_s) {
                broken = true;
                for (auto& p : s.parts) {
                    p.req->in_flight--;
                    fail_locked(p.req, MIDSX_TIMEOUT, "launch exceeded the deadline");
                    unpin_locked(p.req);
                }
                s.parts.clear();
                s.busy = false;  // the slot is abandoned with the server
                changed = true;
            }
            continue;
        }
        changed = true;
        s.busy = false;
        if (q != cudaSuccess) {
            broken = true;
            std::string why = std::string("launch failed: ") + cudaGetErrorString(q);
            for (auto& p : s.parts) {
                p.req->in_flight--;
                fail_locked(p.req, MIDSX_CUDA_ERROR, why);
                unpin_locked(p.req);
            }
            s.parts.clear();
            continue;
        }
        float ms = 0;
        if (cudaEventElapsedTime(&ms, s.start, s.end) == cudaSuccess) st.busy_seconds += ms * 1e-3;
        const double t = now();
        for (auto& p : s.parts) {
            Request* r = p.req;
            r->in_flight--;
            r->done += p.n;
            st.histories += p.n;
            if (r->state == MIDSX_REQ_RUNNING && r->done == r->r.n_histories) {
                r->state = MIDSX_REQ_DONE;
                r->t_done = t;
                st.completed++;
                active.erase(std::remove(active.begin(), active.end(), r), active.end());
                cv_done.notify_all();
            }
            unpin_locked(r);
        }
        s.parts.clear();
    }
    return changed;
}

// Admits queued requests in arrival order while a slot and the budget allow.
bool midsx_gpu_server::admit_locked(bool& enqueued_setup) {
    bool changed = false;
    while (!queue.empty() && int(active.size()) < max_active && !broken) {
        Request* r = queue.front();
        Phantom& ph = *phantoms[size_t(r->r.phantom)];
        size_t need = r->tally_bytes + (ph.dev ? 0 : ph.bytes);
        // evict idle phantoms, least recently used first, until the request fits
        while (st.bytes_in_use + need > budget) {
            Phantom* victim = nullptr;
            for (auto& q : phantoms)
                if (q.get() != &ph && q->dev && q->refs == 0 && (!victim || q->last_use < victim->last_use))
                    victim = q.get();
            if (!victim) break;
            cudaFreeAsync(victim->dev, setup);
            midsx::rt::phantom_bind(victim->h, nullptr);
            victim->dev = nullptr;
            st.bytes_in_use -= victim->bytes;
            st.resident_phantom_bytes -= victim->bytes;
            st.phantom_evictions++;
            enqueued_setup = true;
        }
        if (st.bytes_in_use + need > budget) break;  // wait for releases
        if (!ph.dev) {
            uint8_t* dev = nullptr;
            cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&dev), ph.bytes, pool, setup);
            if (e != cudaSuccess) {
                queue.pop_front();
                fail_locked(r, MIDSX_OOM, std::string("phantom upload: ") + cudaGetErrorString(e));
                changed = true;
                continue;
            }
            e = cudaMemcpyAsync(dev, ph.host.data(), ph.bytes, cudaMemcpyHostToDevice, setup);
            if (e != cudaSuccess) {
                cudaFreeAsync(dev, setup);
                queue.pop_front();
                fail_locked(r, MIDSX_CUDA_ERROR, std::string("phantom upload: ") + cudaGetErrorString(e));
                changed = true;
                continue;
            }
            ph.dev = dev;
            midsx::rt::phantom_bind(ph.h, dev);
            st.bytes_in_use += ph.bytes;
            st.resident_phantom_bytes += ph.bytes;
            st.phantom_uploads++;
            r->footprint += ph.bytes;
        }
        midsx_tallies_h t = nullptr;
        midsx_status s = midsx::rt::tallies_create_async(r->r.dose_mode > 0 ? ph.h : nullptr, r->specs.data(),
                                                         int(r->specs.size()), r->r.dose_mode, pool, setup, &t);
        queue.pop_front();
        enqueued_setup = true;
        changed = true;
        if (s != MIDSX_OK) {
            fail_locked(r, s, midsx::last_error());
            continue;
        }
        midsx::rt::set_tallies_precision(t, r->r.precision);
        r->tallies = t;
        r->footprint += r->tally_bytes;
        st.bytes_in_use += r->tally_bytes;
        st.peak_bytes_in_use = std::max(st.peak_bytes_in_use, st.bytes_in_use);
        ph.refs++;
        r->pinned = true;
        ph.last_use = ++use_clock;
        r->state = MIDSX_REQ_RUNNING;
        r->t_admit = now();
        r->admit_seq = ++admit_counter;
        active.push_back(r);
        st.admitted++;
        st.max_active_seen = std::max<int32_t>(st.max_active_seen, int32_t(active.size()));
    }
    return changed;
}

// Fills free slots with launches over the admitted requests that have histories left.
bool midsx_gpu_server::launch_locked() {
    bool changed = false;
    const size_t rec = midsx::rt::job_record_bytes();
    for (int i = 0; i < n_slots && !broken; ++i) {
        Slot& s = slots[i];
        if (s.busy) continue;
        // A launch runs requests of one (tables, precision) group.  Serve the group of the
        // request that has waited longest since its last launch (then the earliest admitted),
        // so that groups take turns and no request starves behind a long one.
        Request* first = nullptr;
        for (Request* r : active)
            if (r->scheduled < r->r.n_histories &&
                (!first || r->last_launch < first->last_launch ||
                 (r->last_launch == first->last_launch && r->admit_seq < first->admit_seq)))
                first = r;
        if (!first) break;
        const int precision = first->r.precision;
        midsx_tables_h tables = phantoms[size_t(first->r.phantom)]->tables;
        std::vector<Request*> cand;
        for (Request* r : active)
            if (r->r.precision == precision && phantoms[size_t(r->r.phantom)]->tables == tables &&
                r->scheduled < r->r.n_histories && int(cand.size()) < kMaxJobs)
                cand.push_back(r);
        // Size-aware shares.  Three quarters of the launch go to the requests with the fewest
        // histories left, each taking all it needs in turn (shortest remaining first: a small
        // dose request arriving behind 1e8-history radiographs finishes in its first launch);
        // the last quarter, and whatever the small requests left, is shared equally by the
        // requests still short (those that need less than a share take only that), so large
        // requests keep progressing under any load.  Equal shares alone gave a 1e6-history
        // request ~70k histories per launch in a mix of 57 requests: ~14 launches to finish.
        std::vector<Request*> order(cand);
        std::sort(order.begin(), order.end(), [](const Request* a, const Request* b) {
            const uint64_t ra = a->r.n_histories - a->scheduled, rb = b->r.n_histories - b->scheduled;
            return ra < rb || (ra == rb && a->admit_seq < b->admit_seq);
        });
        std::map<Request*, uint64_t> give;
        uint64_t first_h = launch_histories - launch_histories / 4;
        for (Request* r : order) {
            const uint64_t g = std::min(r->r.n_histories - r->scheduled, first_h);
            if (g == 0) break;
            give[r] = g;
            first_h -= g;
        }
        uint64_t budget_h = launch_histories / 4 + first_h;
        std::vector<Request*> rest;
        for (Request* r : order)
            if (r->r.n_histories - r->scheduled > give[r]) rest.push_back(r);
        for (size_t k = 0; k < rest.size(); ++k) {
            const uint64_t rem = rest[k]->r.n_histories - rest[k]->scheduled - give[rest[k]];
            const uint64_t share = std::max<uint64_t>(1, budget_h / uint64_t(rest.size() - k));
            const uint64_t g = std::min(rem, share);
            give[rest[k]] += g;
            budget_h -= std::min(budget_h, g);
        }
        // job records in admission order
        s.parts.clear();
        unsigned long long total = 0;
        s.host_prefix[0] = 0;
        int nj = 0;
        uint32_t step_cap = 0;
        for (Request* r : cand) {
            const uint64_t n = give[r];
            if (n == 0) continue;  // no histories in this launch (the budget went to others)
            uint32_t job_cap = 0;
            midsx_status ps = midsx::rt::pack_job(tables, phantoms[size_t(r->r.phantom)]->h, r->r.source, r->tallies,
                                                  r->r.seed, r->r.first_history + r->scheduled, n, precision,
                                                  s.host_jobs + size_t(nj) * rec, &job_cap);
            if (ps != MIDSX_OK) {
                fail_locked(r, ps, midsx::last_error());
                changed = true;
                continue;
            }
            total += n;
            step_cap = std::max(step_cap, job_cap);
            s.host_prefix[nj + 1] = total;
            s.parts.push_back({r, n});
            ++nj;
        }
        if (nj == 0) continue;
        midsx_run_config c = cfg.launch;
        c.precision = precision;
        bool good = ok(cudaMemcpyAsync(s.dev_jobs, s.host_jobs, size_t(nj) * rec, cudaMemcpyHostToDevice, s.stream),
                       "cudaMemcpyAsync") &&
                    ok(cudaMemcpyAsync(s.dev_prefix, s.host_prefix, size_t(nj + 1) * 8, cudaMemcpyHostToDevice,
                                       s.stream),
                       "cudaMemcpyAsync");
        // every launch waits for the setup work recorded so far (uploads, zeroed tallies): a
        // request admitted in an earlier pass of the scheduler may take its first launch now,
        // while the setup stream is still working through a large upload or memset
        if (good && setup_recorded) good = ok(cudaStreamWaitEvent(s.stream, setup_done, 0), "cudaStreamWaitEvent");
        if (good) good = ok(cudaEventRecord(s.start, s.stream), "cudaEventRecord");
        bool spectra = false;
        for (auto& p : s.parts) spectra |= midsx::rt::tallies_spectra(p.req->tallies);
        midsx_status ls = good ? midsx::rt::launch_packed(tables, s.dev_jobs, nj, s.dev_prefix, total, s.dev_counter, c,
                                                          s.stream, spectra, step_cap)
                               : MIDSX_CUDA_ERROR;
        if (ls == MIDSX_OK) good = ok(cudaEventRecord(s.end, s.stream), "cudaEventRecord");
        if (ls != MIDSX_OK || !good) {
            const std::string why = midsx::last_error();
            for (auto& p : s.parts) fail_locked(p.req, ls != MIDSX_OK ? ls : MIDSX_CUDA_ERROR, why);
            s.parts.clear();
            broken = ls == MIDSX_CUDA_ERROR || !good;
            changed = true;
            continue;
        }
        const double t = now();
        st.launches++;
        for (auto& p : s.parts) {
            Request* r = p.req;
            r->scheduled += p.n;
            r->last_launch = st.launches;
            r->launches++;
            r->in_flight++;
            if (r->t_first < 0) r->t_first = t;
        }
        s.busy = true;
        s.issued = Clock::now();
        changed = true;
    }
    return changed;
}

void midsx_gpu_server::run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        bool changed = retire_locked();
        // memory of released requests goes back to the pool before new admissions
        bool setup_enqueued = false;
        for (auto it = to_free.begin(); it != to_free.end();) {
            Request* r = *it;
            if (r->in_flight > 0) {
                ++it;
                continue;
            }
            free_request_memory_locked(r);
            requests.erase(r->id);
            it = to_free.erase(it);
            setup_enqueued = true;
        }
        if (stop) {
            bool any_busy = false;
            for (int i = 0; i < n_slots; ++i) any_busy |= slots[i].busy;
            if (!any_busy) break;
        } else {
            changed |= admit_locked(setup_enqueued);
            if (setup_enqueued) {
                if (!ok(cudaEventRecord(setup_done, setup), "cudaEventRecord"))
                    broken = true;
                else
                    setup_recorded = true;
            }
            changed |= launch_locked();
        }
        st.queued = int32_t(queue.size());
        st.active = int32_t(active.size());
        if (!changed) {
            bool any_busy = false;
            for (int i = 0; i < n_slots; ++i) any_busy |= slots[i].busy;
            // poll the device while launches run; otherwise sleep until a client acts
            if (any_busy)
                cv_sched.wait_for(lk, std::chrono::microseconds(100));
            else
                cv_sched.wait_for(lk, std::chrono::milliseconds(50));
        }
    }
}

// ============================================================================== C ABI ===
extern "C" midsx_status midsx_server_create(midsx_tables_h tables, const midsx_server_config* cfg,
                                            midsx_server_h* out) {
    if (!tables || !out) return MIDSX_INVALID_ARG;
    auto srv = std::make_unique<midsx_gpu_server>();
    midsx_gpu_server* s = srv.get();
    s->tables = tables;
    s->device = midsx::rt::tables_device(tables);
    if (cfg) s->cfg = *cfg;
    s->launch_histories = s->cfg.launch_histories ? s->cfg.launch_histories : 4000000ull;
    s->max_active = s->cfg.max_active > 0 ? std::min(s->cfg.max_active, kMaxJobs) : kMaxJobs;
    s->n_slots = s->cfg.launches_in_flight > 0 ? std::min(s->cfg.launches_in_flight, kMaxSlots) : 2;
    if (const char* env = std::getenv("MIDSX_WAIT_TIMEOUT_S")) s->deadline_s = std::atof(env);
    if (s->cfg.max_active < 0 || s->cfg.launches_in_flight < 0) {
        midsx::set_last_error("midsx_server_create: negative max_active or launches_in_flight");
        return MIDSX_INVALID_ARG;
    }
    if (!ok(cudaSetDevice(s->device), "cudaSetDevice")) return MIDSX_CUDA_ERROR;
    size_t free_b = 0, total_b = 0;
    if (!ok(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo")) return MIDSX_CUDA_ERROR;
    s->budget = s->cfg.hbm_budget_bytes ? s->cfg.hbm_budget_bytes : uint64_t(double(free_b) * 0.9);
    s->st.budget_bytes = s->budget;

    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    if (!ok(cudaMemPoolCreate(&s->pool, &props), "cudaMemPoolCreate")) return MIDSX_CUDA_ERROR;
    uint64_t keep = ~0ull;  // keep freed blocks in the pool for the next requests
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    bool good = ok(cudaStreamCreateWithFlags(&s->setup, cudaStreamNonBlocking), "cudaStreamCreate") &&
                ok(cudaEventCreateWithFlags(&s->setup_done, cudaEventDisableTiming), "cudaEventCreate");
    const size_t rec = midsx::rt::job_record_bytes();
    for (int i = 0; i < s->n_slots && good; ++i) {
        Slot& sl = s->slots[i];
        good = ok(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking), "cudaStreamCreate") &&
               ok(cudaEventCreate(&sl.start), "cudaEventCreate") && ok(cudaEventCreate(&sl.end), "cudaEventCreate") &&
               ok(cudaMallocHost(reinterpret_cast<void**>(&sl.host_jobs), kMaxJobs * rec), "cudaMallocHost") &&
               ok(cudaMallocHost(reinterpret_cast<void**>(&sl.host_prefix), (kMaxJobs + 1) * 8), "cudaMallocHost") &&
               ok(cudaMalloc(&sl.dev_jobs, kMaxJobs * rec), "cudaMalloc") &&
               ok(cudaMalloc(reinterpret_cast<void**>(&sl.dev_prefix), (kMaxJobs + 1) * 8), "cudaMalloc") &&
               ok(cudaMalloc(reinterpret_cast<void**>(&sl.dev_counter), 8 * (1 + MIDSX_MAX_BATCH_JOBS)), "cudaMalloc");
    }
    s->t0 = Clock::now();
    if (!good) {
        midsx_server_destroy(srv.release());
        return MIDSX_CUDA_ERROR;
    }
    s->worker = std::thread([s] { s->run(); });
    *out = srv.release();
    return MIDSX_OK;
}

extern "C" midsx_status midsx_server_destroy(midsx_server_h s) {
    if (!s) return MIDSX_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_sched.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->device);
    for (auto& kv : s->requests) s->free_request_memory_locked(kv.second.get());
    for (auto& p : s->phantoms) {
        if (p->dev) cudaFreeAsync(p->dev, s->setup);
        if (p->h) midsx::rt::phantom_delete_handle(p->h);
    }
    // after a failed or timed-out launch the device may not answer: do not wait on it
    if (s->setup && !s->broken) cudaStreamSynchronize(s->setup);
    for (int i = 0; i < kMaxSlots; ++i) {
        Slot& sl = s->slots[i];
        if (sl.stream && !s->broken) cudaStreamSynchronize(sl.stream);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.start) cudaEventDestroy(sl.start);
        if (sl.end) cudaEventDestroy(sl.end);
        if (sl.host_jobs) cudaFreeHost(sl.host_jobs);
        if (sl.host_prefix) cudaFreeHost(sl.host_prefix);
        cudaFree(sl.dev_jobs);
        cudaFree(sl.dev_prefix);
        cudaFree(sl.dev_counter);
    }
    if (s->setup_done) cudaEventDestroy(s->setup_done);
    if (s->setup) cudaStreamDestroy(s->setup);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_server_add_phantom(midsx_server_h s, midsx_tables_h tables,
                                                 const midsx_geometry_spec* geom, const uint8_t* ids,
                                                 int32_t* phantom_id) {
    if (!s || !geom || !ids || !phantom_id) return MIDSX_INVALID_ARG;
    if (!tables) tables = s->tables;
    if (midsx::rt::tables_device(tables) != s->device) {
        midsx::set_last_error("midsx_server_add_phantom: tables on another device");
        return MIDSX_INVALID_ARG;
    }
    midsx_phantom_h h = nullptr;
    midsx_status st = midsx_gpu_phantom_create(tables, geom, ids, &h);
    if (st != MIDSX_OK) return st;
    auto p = std::make_unique<Phantom>();
    p->h = h;
    p->tables = tables;
    p->bytes = midsx::rt::phantom_voxels(h);
    st = midsx::rt::phantom_download(h, p->host);
    midsx::rt::phantom_drop_storage(h);  // residency is the server's (pool storage)
    if (st != MIDSX_OK) {
        midsx::rt::phantom_delete_handle(h);
        return st;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    *phantom_id = int32_t(s->phantoms.size());
    s->phantoms.push_back(std::move(p));
    return MIDSX_OK;
}

extern "C" midsx_status midsx_server_submit(midsx_server_h s, const midsx_request* r, uint64_t* request_id) {
    if (!s || !r || !request_id) return MIDSX_INVALID_ARG;
    if (r->precision != MIDSX_PREC_FP64 && r->precision != MIDSX_PREC_MIXED) {
        midsx::set_last_error("midsx_server_submit: unknown precision");
        return MIDSX_INVALID_ARG;
    }
    if (!r->source || r->n_histories == 0 || r->n_tallies < 0 || r->n_tallies > MIDSX_MAX_TALLIES ||
        (r->n_tallies > 0 && !r->tallies) || r->dose_mode < 0 || r->dose_mode > 2) {
        midsx::set_last_error("midsx_server_submit: invalid request");
        return MIDSX_INVALID_ARG;
    }
    auto q = std::make_unique<Request>();
    q->r = *r;
    q->specs.assign(r->tallies, r->tallies + r->n_tallies);
    q->r.tallies = nullptr;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->broken) {
        midsx::set_last_error("midsx_server_submit: the server stopped after a failed launch");
        return MIDSX_CUDA_ERROR;
    }
    if (r->phantom < 0 || size_t(r->phantom) >= s->phantoms.size()) {
        midsx::set_last_error("midsx_server_submit: unknown phantom");
        return MIDSX_NOT_FOUND;
    }
    const Phantom& ph = *s->phantoms[size_t(r->phantom)];
    q->tally_bytes = midsx::rt::tallies_footprint(ph.bytes, q->specs.data(), int(q->specs.size()), r->dose_mode);
    if (q->tally_bytes == 0) return MIDSX_INVALID_ARG;  // tallies_layout set the message
    if (q->tally_bytes + ph.bytes > s->budget) {
        midsx::set_last_error("midsx_server_submit: the request's footprint exceeds the HBM budget");
        return MIDSX_OOM;
    }
    q->id = s->next_id++;
    q->t_submit = s->now();
    *request_id = q->id;
    s->queue.push_back(q.get());
    s->requests[q->id] = std::move(q);
    s->st.submitted++;
    s->cv_sched.notify_all();
    return MIDSX_OK;
}

namespace {

void fill_info(const Request& r, midsx_request_info* out) {
    std::memset(out, 0, sizeof(*out));
    out->state = r.state;
    out->status = r.status;
    out->launches = r.launches;
    out->histories_scheduled = r.scheduled;
    out->histories_done = r.done;
    out->footprint_bytes = r.footprint;
    out->t_submit = r.t_submit;
    out->t_admit = r.t_admit;
    out->t_first_launch = r.t_first;
    out->t_done = r.t_done;
}

}  // namespace

extern "C" midsx_status midsx_server_poll(midsx_server_h s, uint64_t request_id, midsx_request_info* out) {
    if (!s || !out) return MIDSX_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end() || it->second->released) return MIDSX_NOT_FOUND;
    fill_info(*it->second, out);
    if (it->second->state == MIDSX_REQ_FAILED) midsx::set_last_error(it->second->error);
    return MIDSX_OK;
}

extern "C" midsx_status midsx_server_wait(midsx_server_h s, uint64_t request_id, double timeout_s,
                                          midsx_request_info* out) {
    if (!s) return MIDSX_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(
                                       std::max(0.0, timeout_s)));
    for (;;) {
        auto it = s->requests.find(request_id);
        if (it == s->requests.end() || it->second->released) return MIDSX_NOT_FOUND;
        Request& r = *it->second;
        if (r.state == MIDSX_REQ_DONE || r.state == MIDSX_REQ_FAILED) {
            if (out) fill_info(r, out);
            if (r.state == MIDSX_REQ_FAILED) midsx::set_last_error(r.error);
            return MIDSX_OK;
        }
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && Clock::now() >= deadline) {
            if (out) fill_info(r, out);
            midsx::set_last_error("midsx_server_wait: timed out");
            return MIDSX_TIMEOUT;
        }
    }
}

extern "C" midsx_status midsx_server_tallies(midsx_server_h s, uint64_t request_id, midsx_tallies_h* out) {
    if (!s || !out) return MIDSX_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end() || it->second->released) return MIDSX_NOT_FOUND;
    if (it->second->state != MIDSX_REQ_DONE) {
        midsx::set_last_error("midsx_server_tallies: the request is not done");
        return MIDSX_INVALID_ARG;
    }
    *out = it->second->tallies;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_server_release(midsx_server_h s, uint64_t request_id) {
    if (!s) return MIDSX_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end() || it->second->released) return MIDSX_NOT_FOUND;
    Request* r = it->second.get();
    if (r->state == MIDSX_REQ_QUEUED) {
        s->queue.erase(std::remove(s->queue.begin(), s->queue.end(), r), s->queue.end());
        s->requests.erase(it);
        return MIDSX_OK;
    }
    if (r->state == MIDSX_REQ_RUNNING) {
        midsx::set_last_error("midsx_server_release: the request is still running");
        return MIDSX_INVALID_ARG;
    }
    r->released = true;
    if (r->tallies) s->st.bytes_in_use -= r->tally_bytes;
    s->to_free.push_back(r);
    s->cv_sched.notify_all();
    return MIDSX_OK;
}

extern "C" midsx_status midsx_server_get_stats(midsx_server_h s, midsx_server_stats* out) {
    if (!s || !out) return MIDSX_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->queued = int32_t(s->queue.size());
    out->active = int32_t(s->active.size());
    return MIDSX_OK;
}

extern "C" midsx_status midsx_server_now(midsx_server_h s, double* t) {
    if (!s || !t) return MIDSX_INVALID_ARG;
    *t = s->now();
    return MIDSX_OK;
}
