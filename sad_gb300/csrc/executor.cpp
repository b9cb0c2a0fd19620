// executor.cpp -- many fits and renders in flight on one GPU.
//
// The reference fits one image per process (run.sh's batch mode runs the CLI once per
// file, run.sh:262-373).  Small images leave most of a 152-SM GPU idle, so here a pool of
// host worker threads, each with its own CUDA streams, runs requests concurrently:
//   * fit: a trainer placed in one stream-ordered slab (sad_trainer_create_in), the whole
//     schedule, sites and PSNR back to host memory;
//   * render: sites up, candidate field + render (sad_render_from_sites), pixels back;
//   * resident fit sessions: open (a trainer placed in its slab, target up, init), any
//     number of continue requests (more iterations of the same fit -- sites, Adam moments,
//     candidate fields and device counters stay on the device between requests -- then
//     sites and PSNR back), close (the slab freed).  A session's slab counts against the
//     budget from open to close; its requests run one at a time, in submission order.
// Device memory comes from the device's stream-ordered pool (cudaMallocAsync /
// cudaFreeAsync): a request's slab is reused by later requests without a device-wide
// synchronisation (cudaFree would wait for every stream).  Admission is first in, first
// out, and holds a request back while the slabs in use plus its own exceed the budget.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "host_common.h"

namespace {

using Clock = std::chrono::steady_clock;

enum Kind { kFit = 0, kRender = 1, kOpen = 2, kContinue = 3, kClose = 4 };

struct Request {
    uint64_t ticket = 0;
    int kind = 0;  // Kind
    uint64_t session = 0;  // kOpen / kContinue / kClose
    int iterations = 0;    // kContinue
    sad_train_config_t tcfg{};
    sad_render_config_t rcfg{};
    const float* target = nullptr;
    const float* mask = nullptr;
    const float* sites_in = nullptr;
    uint32_t n = 0;
    int w = 0, h = 0;
    float* sites_out = nullptr;
    int capacity = 0;
    float* rgb_out = nullptr;
    sad_request_result_t* result = nullptr;
    size_t need = 0;
    Clock::time_point submitted;
};

inline size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

size_t render_need(const sad_render_config_t& c, uint32_t n, int w, int h) {
    return 256 + a256(size_t(n) * 40) + a256(size_t(w) * h * 12) +
           sad_render_scratch_bytes(n, w, h, c.cand_downscale);
}

void set_message(sad_request_result_t* r, sad_status_t st) {
    r->status = st;
    if (st != SAD_OK) {
        std::strncpy(r->message, sad_last_error(), sizeof(r->message) - 1);
        r->message[sizeof(r->message) - 1] = '\0';
    }
}

// A resident fit: its trainer lives in its slab from open to close.
struct Session {
    sad_trainer_t* trainer = nullptr;
    void* mem = nullptr;
    size_t need = 0;
    int total_iterations = 0;  // the schedule's length (its configuration's iterations)
    bool closing = false;  // a close request is queued: no further requests
    bool opened = false;  // the open request has run (successfully or not)
    bool failed = false;  // the open request failed: later requests report it
    bool busy = false;    // one of its requests is running
    std::string error;
};

}  // namespace

struct sad_executor {
    int device = 0;
    size_t budget = 0;  // 0: no limit
    size_t in_use = 0;
    int max_fits = 0;   // 0: no limit
    int running_fits = 0;
    int inject_slab_failures = 0;  // host-side refusals still to make (failure tests)
    bool stop = false;
    uint64_t next_ticket = 1;
    std::deque<Request> queue;
    std::unordered_set<uint64_t> inflight;  // queued or running
    uint64_t next_session = 1;
    std::unordered_map<uint64_t, Session> sessions;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<std::thread> workers;
};

namespace {

sad_status_t run_fit(const Request& q, void* mem, sad_request_result_t* r) {
    sad::NvtxRange r_nvtx("executor fit request");
    sad_trainer_t* t = nullptr;
    SAD_TRY(sad_trainer_create_in(&q.tcfg, q.w, q.h, mem, q.need, &t));
    int written = 0;
    float psnr = 0.0f;
    sad_status_t st = sad_trainer_fit_host(t, q.target, q.mask, q.sites_out, q.capacity, &written, &psnr);
    sad_trainer_destroy(t);  // synchronises the trainer's streams
    r->sites_written = written;
    r->psnr = psnr;
    return st;
}

sad_status_t run_render(const Request& q, void* mem, cudaStream_t ws) {
    sad::NvtxRange r_nvtx("executor render request");
    char* p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(mem) + 255) & ~uintptr_t(255));
    float* sites = reinterpret_cast<float*>(p);
    p += a256(size_t(q.n) * 40);
    float* rgb = reinterpret_cast<float*>(p);
    size_t npx = size_t(q.w) * q.h;
    p += a256(npx * 12);
    size_t scratch = sad_render_scratch_bytes(q.n, q.w, q.h, q.rcfg.cand_downscale);
    SAD_TRY(sad::check_cuda(cudaMemcpyAsync(sites, q.sites_in, size_t(q.n) * 40, cudaMemcpyHostToDevice, ws),
                            "executor render: sites upload"));
    SAD_TRY(sad_render_from_sites(&q.rcfg, sites, q.n, q.w, q.h, rgb, p, scratch,
                                  reinterpret_cast<sad_stream_t>(ws)));
    SAD_TRY(sad::check_cuda(cudaMemcpyAsync(q.rgb_out, rgb, npx * 12, cudaMemcpyDeviceToHost, ws),
                            "executor render: pixels download"));
    return sad::check_cuda(cudaStreamSynchronize(ws), "executor render: sync");
}

// Session requests run on the session's trainer, outside the executor's lock (the session
// is marked busy, so no other worker touches it meanwhile).
sad_status_t run_open(const Request& q, Session& ss, void* mem, sad_request_result_t* r) {
    sad::NvtxRange r_nvtx("executor open fit session");
    sad_trainer_t* t = nullptr;
    SAD_TRY(sad_trainer_create_in(&q.tcfg, q.w, q.h, mem, q.need, &t));
    sad_status_t st = sad_trainer_set_target_host(t, q.target, q.mask);
    if (st == SAD_OK) st = sad_trainer_init(t, nullptr, 0);
    if (st == SAD_OK) st = sad_trainer_render(t, nullptr, &r->psnr);
    if (st != SAD_OK) {
        sad_trainer_destroy(t);
        return st;
    }
    ss.trainer = t;
    ss.mem = mem;
    return SAD_OK;
}

sad_status_t run_continue(const Request& q, Session& ss, sad_request_result_t* r) {
    sad::NvtxRange r_nvtx("executor continue fit session");
    sad_trainer_info_t info{};
    SAD_TRY(sad_trainer_info(ss.trainer, &info));
    const int end = std::min(ss.total_iterations, info.iteration + std::max(0, q.iterations));
    SAD_TRY(sad_trainer_run(ss.trainer, end));
    SAD_TRY(sad_trainer_render(ss.trainer, nullptr, &r->psnr));
    int written = 0;
    if (q.capacity > 0) SAD_TRY(sad_trainer_get_sites(ss.trainer, q.sites_out, q.capacity, 1, &written));
    r->sites_written = written;
    r->iteration = end;
    return SAD_OK;
}

void worker_main(sad_executor* ex) {
    // a worker whose device or stream cannot be set up still takes requests and fails
    // each with that error, so no waiter is left behind
    cudaStream_t ws = nullptr;
    sad_status_t setup = sad::check_cuda(cudaSetDevice(ex->device), "executor worker: device");
    // the worker's own stream (renders, slab allocation) at the device's highest priority:
    // a render's blocks are scheduled ahead of pending fit blocks as SMs free up, so a
    // short render is not queued behind a fit's kernels
    int least = 0, greatest = 0;
    if (setup == SAD_OK)
        setup = sad::check_cuda(cudaDeviceGetStreamPriorityRange(&least, &greatest), "executor worker: priorities");
    if (setup == SAD_OK)
        setup = sad::check_cuda(cudaStreamCreateWithPriority(&ws, cudaStreamNonBlocking, greatest),
                                "executor worker: stream");
    const std::string setup_error = setup == SAD_OK ? std::string() : std::string(sad_last_error());
    for (;;) {
        Request q;
        bool refused = false;  // slab refused by failure injection
        {
            std::unique_lock<std::mutex> lock(ex->mu);
            // the earliest queued request that fits the memory budget and, for a fit, the
            // cap on running fits (so renders pass fits that wait for a fit slot)
            // (a session's requests wait while another of its requests runs, and follow
            // its open request)
            // Under memory pressure, requests that need memory keep first-in-first-out order
            // behind the first one that does not fit; requests that need none (a session's
            // continue and close) may pass it, so a session can always finish and release.
            std::unordered_set<uint64_t> passed;  // sessions with an earlier queued request
            auto pick = [&]() -> std::deque<Request>::iterator {
                passed.clear();
                bool blocked = false;
                for (auto it = ex->queue.begin(); it != ex->queue.end(); ++it) {
                    if (it->session) {
                        // a request of a session that no longer exists runs (and fails) at once
                        auto ss = ex->sessions.find(it->session);
                        bool ready = ss == ex->sessions.end() ||
                                     (!ss->second.busy && (it->kind == kOpen || ss->second.opened) &&
                                      !passed.count(it->session));
                        passed.insert(it->session);
                        if (!ready) continue;
                    }
                    if (blocked && it->need > 0) continue;
                    bool mem = ex->budget == 0 || ex->in_use == 0 || ex->in_use + it->need <= ex->budget;
                    bool slot = it->kind != kFit || ex->max_fits == 0 || ex->running_fits < ex->max_fits;
                    if (mem && slot) return it;
                    if (!mem) blocked = true;
                }
                return ex->queue.end();
            };
            ex->cv_work.wait(lock, [&] { return pick() != ex->queue.end() || (ex->stop && ex->queue.empty()); });
            if (ex->queue.empty()) break;  // stopped and drained
            auto it = pick();
            q = *it;
            ex->queue.erase(it);
            ex->in_use += q.need;
            if (q.kind == kFit) ++ex->running_fits;
            if (q.session) {
                auto ss = ex->sessions.find(q.session);
                if (ss != ex->sessions.end()) ss->second.busy = true;
            }
            if (ex->inject_slab_failures > 0) {
                --ex->inject_slab_failures;
                refused = true;
            }
        }
        sad_request_result_t* r = q.result;
        Clock::time_point start = Clock::now();
        r->queue_ms = std::chrono::duration<double, std::milli>(start - q.submitted).count();
        sad::clear_error();
        void* mem = nullptr;
        sad_status_t st = setup;
        if (st != SAD_OK) sad::set_error("%s", setup_error.c_str());
        if (st == SAD_OK && refused) {
            sad::set_error("executor: slab allocation refused (injected failure)");
            st = SAD_ERR_OUT_OF_MEMORY;
        }
        Session* ss = nullptr;  // node-stable: unordered_map never moves its elements
        if (q.session) {
            std::lock_guard<std::mutex> lock(ex->mu);
            auto it = ex->sessions.find(q.session);
            if (it != ex->sessions.end()) ss = &it->second;
        }
        if (st == SAD_OK && q.session && !ss) {
            sad::set_error("executor session: closed");
            st = SAD_ERR_INVALID_ARGUMENT;
        }
        if (st == SAD_OK && ss && q.kind == kContinue && ss->failed) {
            sad::set_error("executor session: %s", ss->error.c_str());
            st = SAD_ERR_INVALID_ARGUMENT;
        }
        if (st == SAD_OK && q.need > 0) {
            st = sad::check_cuda(cudaMallocAsync(&mem, q.need, ws), "executor: slab allocation");
            if (st == SAD_OK) st = sad::check_cuda(cudaStreamSynchronize(ws), "executor: slab allocation");
        }
        bool keep_slab = false;  // an opened session keeps its slab and its share of the budget
        size_t release = q.need;
        if (st == SAD_OK) {
            switch (q.kind) {
            case kFit: st = run_fit(q, mem, r); break;
            case kRender: st = run_render(q, mem, ws); break;
            case kOpen:
                st = run_open(q, *ss, mem, r);
                keep_slab = st == SAD_OK;
                break;
            case kContinue: st = run_continue(q, *ss, r); break;
            case kClose:
                // the slab (and its share of the budget) is held only after a successful open
                release = ss->trainer ? ss->need : 0;
                if (ss->trainer) sad_trainer_destroy(ss->trainer);  // synchronises its streams
                ss->trainer = nullptr;
                mem = ss->mem;  // freed below
                ss->mem = nullptr;
                break;
            }
        }
        set_message(r, st);
        if (mem && !keep_slab) {
            cudaFreeAsync(mem, ws);
            cudaStreamSynchronize(ws);
        }
        r->run_ms = std::chrono::duration<double, std::milli>(Clock::now() - start).count();
        {
            std::lock_guard<std::mutex> lock(ex->mu);
            if (!keep_slab) ex->in_use -= release;
            if (q.kind == kFit) --ex->running_fits;
            if (ss) {
                ss->busy = false;
                if (q.kind == kOpen) {
                    ss->opened = true;
                    if (st != SAD_OK) {
                        ss->failed = true;
                        ss->error = r->message;
                    }
                }
                if (q.kind == kClose && st == SAD_OK) ex->sessions.erase(q.session);
            }
            ex->inflight.erase(q.ticket);
        }
        ex->cv_done.notify_all();
        ex->cv_work.notify_all();
    }
    if (ws) cudaStreamDestroy(ws);
}

sad_status_t enqueue(sad_executor_t* ex, Request&& q, uint64_t* ticket) {
    {
        std::lock_guard<std::mutex> lock(ex->mu);
        SAD_REQUIRE(!ex->stop, "sad_executor: destroyed");
        q.ticket = ex->next_ticket++;
        q.submitted = Clock::now();
        if (ticket) *ticket = q.ticket;
        ex->inflight.insert(q.ticket);
        ex->queue.push_back(std::move(q));
    }
    ex->cv_work.notify_all();
    return SAD_OK;
}

}  // namespace

extern "C" void sad_executor_config_default(sad_executor_config_t* cfg) {
    if (!cfg) return;
    cfg->workers = 8;
    cfg->hbm_budget_bytes = 0;
    cfg->max_running_fits = 0;
}

extern "C" sad_status_t sad_executor_create(const sad_executor_config_t* cfg, sad_executor_t** out) {
    sad::clear_error();
    SAD_REQUIRE(cfg && out, "sad_executor_create: null argument");
    SAD_REQUIRE(cfg->workers > 0 && cfg->workers <= 256, "sad_executor_create: workers must be 1..256");
    *out = nullptr;
    auto* ex = new sad_executor();
    ex->budget = cfg->hbm_budget_bytes;
    ex->max_fits = cfg->max_running_fits > 0 ? cfg->max_running_fits : 0;
    sad_status_t st = sad::check_cuda(cudaGetDevice(&ex->device), "sad_executor_create: device");
    if (st == SAD_OK) {
        // keep freed slabs in the pool between requests instead of returning them to the
        // driver at every synchronisation (a process-local setting of this device's pool)
        cudaMemPool_t pool = nullptr;
        st = sad::check_cuda(cudaDeviceGetDefaultMemPool(&pool, ex->device), "sad_executor_create: pool");
        uint64_t keep = ex->budget ? ex->budget : ~uint64_t(0);
        if (st == SAD_OK)
            st = sad::check_cuda(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep),
                                 "sad_executor_create: pool threshold");
    }
    if (st != SAD_OK) {
        delete ex;
        return st;
    }
    for (int i = 0; i < cfg->workers; ++i) ex->workers.emplace_back(worker_main, ex);
    *out = ex;
    return SAD_OK;
}

extern "C" sad_status_t sad_executor_submit_fit(sad_executor_t* ex, const sad_train_config_t* cfg,
                                                const float* target_host, const float* mask_host, int width,
                                                int height, float* sites_host, int capacity,
                                                sad_request_result_t* result, uint64_t* ticket) {
    sad::clear_error();
    SAD_REQUIRE(ex && cfg && target_host && result, "sad_executor_submit_fit: null argument");
    SAD_REQUIRE(capacity == 0 || sites_host, "sad_executor_submit_fit: null sites buffer");
    size_t need = sad_trainer_memory_bytes(cfg, width, height);
    SAD_REQUIRE(need > 0, "sad_executor_submit_fit: invalid configuration or size");
    std::memset(result, 0, sizeof(*result));
    Request q;
    q.kind = 0;
    q.tcfg = *cfg;
    q.target = target_host;
    q.mask = mask_host;
    q.w = width;
    q.h = height;
    q.sites_out = sites_host;
    q.capacity = capacity;
    q.result = result;
    q.need = need;
    return enqueue(ex, std::move(q), ticket);
}

extern "C" sad_status_t sad_executor_submit_render(sad_executor_t* ex, const sad_render_config_t* cfg,
                                                   const float* sites_host, uint32_t site_count, int width,
                                                   int height, float* rgb_host, sad_request_result_t* result,
                                                   uint64_t* ticket) {
    sad::clear_error();
    SAD_REQUIRE(ex && cfg && sites_host && rgb_host && result, "sad_executor_submit_render: null argument");
    SAD_REQUIRE(site_count > 0 && sad::image_size_ok(width, height), "sad_executor_submit_render: no sites or invalid image size");
    SAD_REQUIRE(cfg->candidate_passes >= 0, "sad_executor_submit_render: negative candidate passes");
    std::memset(result, 0, sizeof(*result));
    Request q;
    q.kind = 1;
    q.rcfg = *cfg;
    q.sites_in = sites_host;
    q.n = site_count;
    q.w = width;
    q.h = height;
    q.rgb_out = rgb_host;
    q.result = result;
    q.need = render_need(*cfg, site_count, width, height);
    return enqueue(ex, std::move(q), ticket);
}

extern "C" sad_status_t sad_executor_open_fit(sad_executor_t* ex, const sad_train_config_t* cfg,
                                              const float* target_host, const float* mask_host, int width,
                                              int height, sad_request_result_t* result, uint64_t* session,
                                              uint64_t* ticket) {
    sad::clear_error();
    SAD_REQUIRE(ex && cfg && target_host && result && session, "sad_executor_open_fit: null argument");
    size_t need = sad_trainer_memory_bytes(cfg, width, height);
    SAD_REQUIRE(need > 0, "sad_executor_open_fit: invalid configuration or size");
    std::memset(result, 0, sizeof(*result));
    Request q;
    q.kind = kOpen;
    q.tcfg = *cfg;
    q.target = target_host;
    q.mask = mask_host;
    q.w = width;
    q.h = height;
    q.result = result;
    q.need = need;
    {
        std::lock_guard<std::mutex> lock(ex->mu);
        SAD_REQUIRE(!ex->stop, "sad_executor: destroyed");
        q.session = ex->next_session++;
        Session& ss = ex->sessions[q.session];
        ss.need = need;
        ss.total_iterations = cfg->iterations;
    }
    *session = q.session;
    return enqueue(ex, std::move(q), ticket);
}

// Queues a continue or close request of a live session (one whose close is not queued).
static sad_status_t session_request(sad_executor_t* ex, uint64_t session, Request&& q, uint64_t* ticket,
                                    const char* who) {
    {
        std::lock_guard<std::mutex> lock(ex->mu);
        auto it = ex->sessions.find(session);
        if (it == ex->sessions.end() || it->second.closing) {
            sad::set_error("%s: unknown or closed session", who);
            return SAD_ERR_INVALID_ARGUMENT;
        }
        if (q.kind == kClose) it->second.closing = true;
    }
    q.session = session;
    return enqueue(ex, std::move(q), ticket);
}

extern "C" sad_status_t sad_executor_submit_continue(sad_executor_t* ex, uint64_t session, int iterations,
                                                     float* sites_host, int capacity,
                                                     sad_request_result_t* result, uint64_t* ticket) {
    sad::clear_error();
    SAD_REQUIRE(ex && result, "sad_executor_submit_continue: null argument");
    SAD_REQUIRE(iterations >= 0, "sad_executor_submit_continue: negative iterations");
    SAD_REQUIRE(capacity == 0 || sites_host, "sad_executor_submit_continue: null sites buffer");
    std::memset(result, 0, sizeof(*result));
    Request q;
    q.kind = kContinue;
    q.iterations = iterations;
    q.sites_out = sites_host;
    q.capacity = capacity;
    q.result = result;
    q.need = 0;
    return session_request(ex, session, std::move(q), ticket, "sad_executor_submit_continue");
}

extern "C" sad_status_t sad_executor_close_fit(sad_executor_t* ex, uint64_t session, sad_request_result_t* result,
                                               uint64_t* ticket) {
    sad::clear_error();
    SAD_REQUIRE(ex && result, "sad_executor_close_fit: null argument");
    std::memset(result, 0, sizeof(*result));
    Request q;
    q.kind = kClose;
    q.result = result;
    q.need = 0;
    return session_request(ex, session, std::move(q), ticket, "sad_executor_close_fit");
}

extern "C" sad_status_t sad_executor_wait(sad_executor_t* ex, uint64_t ticket) {
    sad::clear_error();
    SAD_REQUIRE(ex, "sad_executor_wait: null executor");
    std::unique_lock<std::mutex> lock(ex->mu);
    SAD_REQUIRE(ticket > 0 && ticket < ex->next_ticket, "sad_executor_wait: unknown ticket");
    ex->cv_done.wait(lock, [&] { return ex->inflight.count(ticket) == 0; });
    return SAD_OK;
}

extern "C" sad_status_t sad_executor_wait_all(sad_executor_t* ex) {
    sad::clear_error();
    SAD_REQUIRE(ex, "sad_executor_wait_all: null executor");
    std::unique_lock<std::mutex> lock(ex->mu);
    ex->cv_done.wait(lock, [&] { return ex->inflight.empty(); });
    return SAD_OK;
}

extern "C" sad_status_t sad_executor_cancel(sad_executor_t* ex, uint64_t ticket, int* cancelled) {
    sad::clear_error();
    SAD_REQUIRE(ex && cancelled, "sad_executor_cancel: null argument");
    *cancelled = 0;
    {
        std::lock_guard<std::mutex> lock(ex->mu);
        SAD_REQUIRE(ticket > 0 && ticket < ex->next_ticket, "sad_executor_cancel: unknown ticket");
        auto it = std::find_if(ex->queue.begin(), ex->queue.end(),
                               [&](const Request& q) { return q.ticket == ticket; });
        if (it == ex->queue.end()) return SAD_OK;  // running or done
        sad_request_result_t* r = it->result;
        r->status = SAD_ERR_CANCELLED;
        std::strncpy(r->message, "cancelled before it started", sizeof(r->message) - 1);
        r->message[sizeof(r->message) - 1] = '\0';
        r->queue_ms = std::chrono::duration<double, std::milli>(Clock::now() - it->submitted).count();
        ex->queue.erase(it);
        ex->inflight.erase(ticket);
        *cancelled = 1;
    }
    ex->cv_done.notify_all();
    ex->cv_work.notify_all();  // the new queue head may fit where the withdrawn one did not
    return SAD_OK;
}

extern "C" sad_status_t sad_executor_inject_slab_failures(sad_executor_t* ex, int count) {
    sad::clear_error();
    SAD_REQUIRE(ex && count >= 0, "sad_executor_inject_slab_failures: invalid argument");
    std::lock_guard<std::mutex> lock(ex->mu);
    ex->inject_slab_failures = count;
    return SAD_OK;
}

extern "C" sad_status_t sad_executor_destroy(sad_executor_t* ex) {
    if (!ex) return SAD_OK;
    {
        std::lock_guard<std::mutex> lock(ex->mu);
        ex->stop = true;  // queued requests still run
    }
    ex->cv_work.notify_all();
    for (auto& t : ex->workers) t.join();
    delete ex;
    return SAD_OK;
}
