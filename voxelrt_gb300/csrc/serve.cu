// serve.cu - request server: continuous batching of render requests over
// resident worlds, edits between frames, admission by an HBM budget, latency stats.
//
// The reference renders one view per frame on the main thread and applies brush
// edits between frames (Main.cpp:83-130, 229-256).  Here many clients submit
// requests concurrently; a scheduler thread packs queued renders into persistent
// launches (vrt_batch's kernel) on up to max_inflight streams, so requests that
// arrive while others run start as soon as a slot and budget free up and their
// work overlaps on the device.  Completion is signalled by a host callback queued
// after each launch's copies, so no thread polls the device.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch_internal.h"
#include "freelist.h"
#include "world.h"

namespace vrt {

namespace {

constexpr uint64_t kPageBytes = 64 * 1024;  // output-arena allocation unit
constexpr uint64_t kPageRecords = kPageBytes / sizeof(vrt_hit);

struct Request {
    uint64_t id = 0;
    uint32_t kind = 0;  // 0 render, 1 edit
    uint32_t state = VRT_REQ_QUEUED;
    vrt_status status = VRT_OK;
    vrt_view view{};
    vrt_hit* host_out = nullptr;
    uint64_t records = 0;
    uint32_t pages = 0, page_base = 0;  // output arena allocation (1-based, 0 = none)
    uint32_t world = 0;
    std::vector<vrt_edit> edits;
    uint32_t batch_size = 0;
    double submit_us = 0, start_us = 0, done_us = 0;
    std::string error;  // why the request failed (the scheduler thread's error text)
};

struct Slot {
    cudaStream_t stream = nullptr;
    DevBuf views, chunk_base, queue;
    ViewDev* h_views = nullptr;  // pinned staging
    uint32_t* h_cb = nullptr;
    size_t staged_cap = 0;
    // recorded after a launch's copies; its status, not the stream's, says whether the
    // launch succeeded (the stream is still busy with the completion callback itself)
    cudaEvent_t done = nullptr;
    std::vector<Request*> reqs;
    bool busy = false;
    std::atomic<bool> complete{false};
    struct vrt_server* server = nullptr;
};

// One resident launch (VRT_SERVE_RESIDENT): the persistent kernel claims the views the
// scheduler publishes through `mailbox` while it runs.  View slots are not reused
// within a launch; a launch takes at most `cap` views.
struct Resident {
    cudaStream_t stream = nullptr;  // the launch
    cudaStream_t ctl = nullptr;     // view uploads
    // records to the host, slot s on copy[s % 4], so that a small view's copy need not
    // queue behind a large one (they share the link's bandwidth)
    cudaStream_t copy[4] = {};
    cudaEvent_t ended = nullptr;
    DevBuf views, chunk_base, remaining, queue;
    unsigned long long* mailbox = nullptr;  // pinned, mapped: the word, then the done flags
    uint32_t* done = nullptr;
    unsigned long long* d_mailbox = nullptr;
    uint32_t* d_done = nullptr;
    ViewDev* h_views = nullptr;  // pinned staging
    uint32_t* h_cb = nullptr;
    uint32_t* h_rem = nullptr;
    unsigned long long* h_hint = nullptr;  // pinned staging of the hint words, one per publish or close
    uint32_t n_hints = 0;                  // staging entries used by the current launch
    uint32_t cap = 0;
    bool live = false, closing = false;
    uint32_t mode = 0;  // traversal mode of the launch's views (view_mode)
    bool full = false;  // the launch takes views with the GPU renderer's whole path
    uint32_t n_views = 0, n_chunks = 0;
    uint32_t first_open = 0;       // slots below it are all finished
    std::vector<Request*> req;     // per view slot
    std::vector<uint8_t> state;    // per slot: 0 tracing, 1 copy issued, 2 finished
    std::vector<cudaEvent_t> copy_ev;
    BatchParams params{};
};
constexpr uint32_t kResidentViews = 4096;

// A request the resident scheduler saw finish, collected before it takes the server lock.
struct Finished {
    Request* r;
    vrt_status status;
    double t;
    std::string error;
};

double now_us(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace
}  // namespace vrt

using namespace vrt;

struct vrt_server {
    int device = 0;
    std::vector<vrt_world*> worlds;
    vrt_server_config cfg{};
    vrt_batch_config bcfg{};
    // persistent grid per traversal mode (view_mode: 0, GLSL, GLSL + anisotropic) of the
    // instantiation the server launches in its scheduling mode: blocks, threads
    int grid[3][2] = {};
    const int* grid_of(uint32_t mode) const {
        return grid[(mode & VRT_VIEW_GLSL_ANISO) ? 2 : (mode & VRT_VIEW_GLSL) ? 1 : 0];
    }
    DevWorld* d_worlds = nullptr;
    uint8_t* arena = nullptr;  // output records of admitted requests
    FreeList pages;
    cudaStream_t edit_stream = nullptr;
    std::vector<std::unique_ptr<Slot>> slots;
    Resident res;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    std::mutex mu;  // queue, requests, stats
    std::condition_variable done_cv;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t next_id = 1;
    uint64_t outstanding = 0;
    bool stop = false;
    bool resident = false;  // scheduling mode (VRT_SERVE_RESIDENT)
    std::thread worker;

    std::mutex sig_mu;  // worker wake-ups (submissions, completions)
    std::condition_variable sig_cv;
    std::atomic<uint64_t> signals{0};

    // stats
    std::vector<double> lat;
    uint64_t renders_done = 0, edits_done = 0, rejected = 0, launches = 0, records_done = 0;
    double busy_since = -1, busy_total = 0;
    int busy_slots = 0;

    void signal() {
        {
            std::lock_guard<std::mutex> g(sig_mu);
            signals++;
        }
        sig_cv.notify_one();
    }
};

namespace {

void CUDART_CB slot_done_cb(void* p) {
    auto* s = static_cast<Slot*>(p);
    s->complete.store(true);
    s->server->signal();
}

vrt_status refresh_world_table(vrt_server* sv) {
    std::vector<DevWorld> t(sv->worlds.size());
    for (size_t i = 0; i < t.size(); i++) t[i] = sv->worlds[i]->dev();
    VRT_CUDA(cudaMemcpy(sv->d_worlds, t.data(), t.size() * sizeof(DevWorld), cudaMemcpyHostToDevice));
    return VRT_OK;
}

void finish(vrt_server* sv, Request* r, vrt_status st, double t) {
    r->status = st;
    if (st != VRT_OK) r->error = last_error_cstr();
    r->state = st == VRT_OK ? VRT_REQ_DONE : VRT_REQ_FAILED;
    r->done_us = t;
    if (r->pages) {
        sv->pages.free(r->page_base, r->pages);
        r->pages = 0;
    }
    if (r->kind == 0) {
        if (st == VRT_OK) {
            sv->lat.push_back(r->done_us - r->submit_us);
            sv->renders_done++;
            sv->records_done += r->records;
        }
    } else {
        sv->edits_done++;
    }
    sv->outstanding--;
}

// Launch the render requests `rs` on slot `s` (called with sv->mu held).
vrt_status launch_slot(vrt_server* sv, Slot& s, std::vector<Request*>& rs) {
    std::vector<vrt_view> views(rs.size());
    for (size_t i = 0; i < rs.size(); i++) views[i] = rs[i]->view;
    LaunchPlan plan;
    const int* g = sv->grid_of(view_mode(views[0]));
    vrt_status st = plan_views(views.data(), (uint32_t)views.size(), (uint32_t)sv->worlds.size(), sv->bcfg, plan,
                               (uint64_t)g[0] * (g[1] / 32));
    if (st != VRT_OK) return st;
    // each request writes into its own arena pages
    for (size_t i = 0; i < rs.size(); i++) plan.views[i].out_base = (uint64_t)(rs[i]->page_base - 1) * kPageRecords;
    const size_t nv = plan.views.size();
    if (s.staged_cap < nv) {
        if (s.h_views) cudaFreeHost(s.h_views);
        if (s.h_cb) cudaFreeHost(s.h_cb);
        s.h_views = nullptr;
        s.h_cb = nullptr;
        const size_t cap = std::max<size_t>(nv, 64);
        VRT_CUDA(cudaHostAlloc(&s.h_views, cap * sizeof(ViewDev), cudaHostAllocDefault));
        VRT_CUDA(cudaHostAlloc(&s.h_cb, (cap + 1) * sizeof(uint32_t), cudaHostAllocDefault));
        s.staged_cap = cap;
    }
    std::memcpy(s.h_views, plan.views.data(), nv * sizeof(ViewDev));
    std::memcpy(s.h_cb, plan.chunk_base.data(), (nv + 1) * sizeof(uint32_t));
    VRT_CUDA(s.views.reserve(nv * sizeof(ViewDev)));
    VRT_CUDA(s.chunk_base.reserve((nv + 1) * sizeof(uint32_t)));
    VRT_CUDA(cudaMemcpyAsync(s.views.ptr, s.h_views, nv * sizeof(ViewDev), cudaMemcpyHostToDevice, s.stream));
    VRT_CUDA(cudaMemcpyAsync(s.chunk_base.ptr, s.h_cb, (nv + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice,
                             s.stream));
    BatchParams p = make_params(plan, sv->d_worlds, (const ViewDev*)s.views.ptr, (const uint32_t*)s.chunk_base.ptr,
                                (uint32_t*)s.queue.ptr, (vrt_hit*)sv->arena);
    if ((st = launch_persistent(p, g[0], g[1], false, s.stream)) != VRT_OK) return st;
    for (size_t i = 0; i < rs.size(); i++) {
        const Request* r = rs[i];
        VRT_CUDA(cudaMemcpyAsync(r->host_out, sv->arena + plan.views[i].out_base * sizeof(vrt_hit),
                                 r->records * sizeof(vrt_hit), cudaMemcpyDeviceToHost, s.stream));
    }
    s.complete.store(false);
    VRT_CUDA(cudaEventRecord(s.done, s.stream));
    VRT_CUDA(cudaLaunchHostFunc(s.stream, slot_done_cb, &s));
    return VRT_OK;
}

void worker_main(vrt_server* sv) {
    cudaSetDevice(sv->device);
    uint64_t seen = 0;
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        bool progressed = false;
        const double t = now_us(sv->t0);
        // retire finished launches
        for (auto& sp : sv->slots) {
            Slot& s = *sp;
            if (!s.busy || !s.complete.load()) continue;
            // the event completed before the callback ran, so it reports the launch's
            // own status (or a sticky error), never "not ready"
            cudaError_t e = cudaEventQuery(s.done);
            if (e == cudaErrorNotReady) continue;
            const vrt_status st = e == cudaSuccess ? VRT_OK : cuda_fail(e, "server launch");
            for (Request* r : s.reqs) finish(sv, r, st, t);
            s.reqs.clear();
            s.busy = false;
            if (--sv->busy_slots == 0 && sv->busy_since >= 0) {
                sv->busy_total += t - sv->busy_since;
                sv->busy_since = -1;
            }
            progressed = true;
        }
        if (progressed) sv->done_cv.notify_all();
        if (sv->stop && sv->queue.empty() && sv->busy_slots == 0) break;
        // an edit runs once nothing is in flight (between frames)
        if (!sv->queue.empty() && sv->queue.front()->kind == 1) {
            if (sv->busy_slots == 0) {
                Request* r = sv->queue.front();
                sv->queue.pop_front();
                r->state = VRT_REQ_RUNNING;
                r->start_us = now_us(sv->t0);
                lk.unlock();
                vrt_status st = vrt_world_edit(sv->worlds[r->world], r->edits.data(), (uint32_t)r->edits.size(),
                                               sv->edit_stream);
                if (st == VRT_OK) st = vrt_world_wait(sv->worlds[r->world]);  // applied before later launches
                if (st == VRT_OK) st = refresh_world_table(sv);
                lk.lock();
                finish(sv, r, st, now_us(sv->t0));
                sv->done_cv.notify_all();
                continue;
            }
        } else if (!sv->queue.empty()) {
            Slot* free_slot = nullptr;
            for (auto& sp : sv->slots)
                if (!sp->busy) {
                    free_slot = sp.get();
                    break;
                }
            if (free_slot) {
                std::vector<Request*> rs;
                while (!sv->queue.empty() && sv->queue.front()->kind == 0 && rs.size() < sv->cfg.max_batch_requests) {
                    Request* r = sv->queue.front();
                    if (!rs.empty() && view_mode(r->view) != view_mode(rs[0]->view)) break;  // one mode per launch
                    const uint32_t base = sv->pages.realloc(0, 0, r->pages);
                    if (base == 0) break;  // budget full: wait for launches to retire
                    r->page_base = base;
                    sv->queue.pop_front();
                    rs.push_back(r);
                }
                if (!rs.empty()) {
                    const double ts = now_us(sv->t0);
                    for (Request* r : rs) {
                        r->state = VRT_REQ_RUNNING;
                        r->start_us = ts;
                        r->batch_size = (uint32_t)rs.size();
                    }
                    free_slot->reqs = rs;
                    free_slot->busy = true;
                    if (sv->busy_slots++ == 0) sv->busy_since = ts;
                    sv->launches++;
                    vrt_status st = launch_slot(sv, *free_slot, rs);
                    if (st != VRT_OK) {
                        cudaStreamSynchronize(free_slot->stream);
                        for (Request* r : rs) finish(sv, r, st, now_us(sv->t0));
                        free_slot->reqs.clear();
                        free_slot->busy = false;
                        sv->busy_slots--;
                        sv->done_cv.notify_all();
                    }
                    continue;
                }
            }
        }
        // sleep until a submission or a completion (1 ms safety net)
        lk.unlock();
        {
            std::unique_lock<std::mutex> g(sv->sig_mu);
            sv->sig_cv.wait_for(g, std::chrono::milliseconds(1), [&] { return sv->signals != seen; });
            seen = sv->signals;
        }
        lk.lock();
    }
}

// ---- resident mode -----------------------------------------------------------------

// Launch configuration of resident launches: one tile per queue chunk, so a single
// request spreads over as many warps as it has tiles.
vrt_batch_config resident_config(const vrt_server* sv) {
    vrt_batch_config cfg = sv->bcfg;
    cfg.chunk_tiles = 1;
    return cfg;
}

bool resident_done_flag(const Resident& R, uint32_t slot) {
    return __atomic_load_n(R.done + slot, __ATOMIC_ACQUIRE) != 0;
}

// The device copy of the mailbox word (8 bytes into the queue block), after a change.
// Stream-ordered behind the view uploads of the same publish, so it lands after them;
// each change stages its own word (no staging memory is reused within a launch, so
// nothing waits for the copies).
void resident_hint(Resident& R, unsigned long long word) {
    unsigned long long* h = R.h_hint + std::min<uint32_t>(R.n_hints++, 2 * R.cap);
    *h = word;
    cudaMemcpyAsync((uint8_t*)R.queue.ptr + kResidentHintOffset, h, 8, cudaMemcpyHostToDevice, R.ctl);
}

// Close the launch's mailbox from the host (the kernel may have closed it already).
void resident_close(Resident& R) {
    unsigned long long cur = __atomic_load_n(R.mailbox, __ATOMIC_ACQUIRE);
    while (!(cur & kMailboxClosed))
        if (__atomic_compare_exchange_n(R.mailbox, &cur, cur | kMailboxClosed, false, __ATOMIC_SEQ_CST,
                                        __ATOMIC_SEQ_CST))
            break;
    R.closing = true;
    if (R.live) resident_hint(R, cur | kMailboxClosed);
}

// Lay out `rs` behind the views already published and publish them: advance the
// mailbox word with one CAS, then enqueue the uploads of the view entries, chunk
// bases and pixel counts and, behind them on the same stream, the device hint the
// warps claim from.  Returns false (nothing published) when the launch was closed
// meanwhile.  No host wait: staging entries belong to their view slot.
bool resident_publish(vrt_server* sv, const std::vector<Request*>& rs, vrt_status& st) {
    Resident& R = sv->res;
    std::vector<vrt_view> views(rs.size());
    for (size_t i = 0; i < rs.size(); i++) views[i] = rs[i]->view;
    LaunchPlan plan;
    st = plan_views(views.data(), (uint32_t)views.size(), (uint32_t)sv->worlds.size(), resident_config(sv), plan);
    if (st != VRT_OK) return false;
    if ((uint64_t)R.n_chunks + plan.chunks >= 0x7fffffffull) {
        resident_close(R);
        return false;
    }
    const uint32_t base = R.n_views, n = (uint32_t)rs.size();
    unsigned long long expected = mailbox_word(R.n_chunks, R.n_views);
    if (!__atomic_compare_exchange_n(R.mailbox, &expected, mailbox_word(R.n_chunks + plan.chunks, base + n), false,
                                     __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
        R.closing = true;  // a warp closed the launch: these requests go to the next one
        return false;
    }
    for (uint32_t i = 0; i < n; i++) {
        ViewDev d = plan.views[i];
        d.chunk_base += R.n_chunks;
        d.out_base = (uint64_t)(rs[i]->page_base - 1) * kPageRecords;
        R.h_views[base + i] = d;
        R.h_cb[base + i] = d.chunk_base;
        R.h_rem[base + i] = d.width * d.height;
        __atomic_store_n(R.done + base + i, 0u, __ATOMIC_RELAXED);
    }
    cudaError_t e = cudaMemcpyAsync((ViewDev*)R.views.ptr + base, R.h_views + base, n * sizeof(ViewDev),
                                    cudaMemcpyHostToDevice, R.ctl);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync((uint32_t*)R.chunk_base.ptr + base, R.h_cb + base, n * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, R.ctl);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync((uint32_t*)R.remaining.ptr + base, R.h_rem + base, n * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, R.ctl);
    if (e != cudaSuccess) {
        // counted in the mailbox but not uploaded: the warps claim from the hint, so
        // close the hint at the count before this publish (no warp reaches these
        // chunks) and the mailbox itself; the requests fail
        st = cuda_fail(e, "resident publish");
        resident_hint(R, mailbox_word(R.n_chunks, R.n_views) | kMailboxClosed);
        unsigned long long cur = __atomic_load_n(R.mailbox, __ATOMIC_ACQUIRE);
        while (!(cur & kMailboxClosed) && !__atomic_compare_exchange_n(R.mailbox, &cur, cur | kMailboxClosed, false,
                                                                      __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
        }
        R.closing = true;
        return false;
    }
    for (uint32_t i = 0; i < n; i++) {
        R.req[base + i] = rs[i];
        R.state[base + i] = 0;
    }
    R.n_views = base + n;
    R.n_chunks += plan.chunks;
    resident_hint(R, mailbox_word(R.n_chunks, R.n_views));
    return true;
}

vrt_status resident_start(vrt_server* sv, uint32_t mode, bool full) {
    const bool glsl = (mode & VRT_VIEW_GLSL) != 0;
    Resident& R = sv->res;
    R.n_views = R.n_chunks = R.first_open = 0;
    R.closing = false;
    R.mode = mode;
    R.full = full;
    R.n_hints = 0;
    VRT_CUDA(cudaStreamSynchronize(R.ctl));  // staging of the last launch is free again
    __atomic_store_n(R.mailbox, 0ull, __ATOMIC_SEQ_CST);
    VRT_CUDA(cudaMemsetAsync(R.queue.ptr, 0, kResidentHintOffset + 8, R.ctl));  // claim counter, counters, hint
    LaunchPlan plan;
    vrt_batch_config cfg = resident_config(sv);
    // fields the config leaves to the library, for a launch whose views arrive later
    resolve_batch_defaults(cfg, nullptr, 0, 0);
    plan.cfg = cfg;
    uint32_t r = 0;
    while ((1u << r) < cfg.tile_w) r++;
    plan.tile_w_log2 = r;
    r = 0;
    while ((1u << r) < cfg.tile_w * cfg.tile_h) r++;
    plan.tile_size_log2 = r;
    plan.glsl = glsl;
    plan.aniso = (mode & VRT_VIEW_GLSL_ANISO) != 0;
    plan.full = full;  // this launch takes views with the GPU renderer's whole path
    BatchParams p = make_params(plan, sv->d_worlds, (const ViewDev*)R.views.ptr, (const uint32_t*)R.chunk_base.ptr,
                                (uint32_t*)R.queue.ptr, (vrt_hit*)sv->arena);
    p.mailbox = R.d_mailbox;
    p.next_chunk = (uint32_t*)R.queue.ptr;
    p.hint = (const unsigned long long*)((uint8_t*)R.queue.ptr + kResidentHintOffset);
    p.remaining = (uint32_t*)R.remaining.ptr;
    p.done_flags = R.d_done;
    p.idle_us = sv->cfg.idle_us;
    p.n_worlds = (uint32_t)sv->worlds.size();
    p.out_records = (unsigned long long)sv->pages.capacity() * kPageRecords;
    R.params = p;
    return VRT_OK;
}

vrt_status resident_launch(vrt_server* sv) {
    Resident& R = sv->res;
    const int* g = sv->grid_of(R.mode);
    vrt_status st = launch_resident(R.params, g[0], g[1], R.stream);
    if (st != VRT_OK) return st;
    VRT_CUDA(cudaEventRecord(R.ended, R.stream));
    R.live = true;
    sv->launches++;
    return VRT_OK;
}

// Copies of finished views, completed copies, the end of the launch.  True if any
// request changed state.
// Collects into `out` the views whose records reached host memory, or that failed,
// without the server lock: slot state belongs to the scheduler thread.  Returns true
// when the launch was seen to end.
bool resident_poll(vrt_server* sv, std::vector<Finished>& out) {
    Resident& R = sv->res;
    auto fail = [&](uint32_t s, vrt_status st) {
        out.push_back({R.req[s], st, now_us(sv->t0), last_error_cstr()});
        R.state[s] = 2;
    };
    while (R.first_open < R.n_views && R.state[R.first_open] == 2) R.first_open++;
    for (uint32_t s = R.first_open; s < R.n_views; s++) {
        if (R.state[s] == 0 && resident_done_flag(R, s)) {
            const Request* r = R.req[s];
            cudaError_t e = cudaMemcpyAsync(r->host_out, sv->arena + (uint64_t)(r->page_base - 1) * kPageBytes,
                                            r->records * sizeof(vrt_hit), cudaMemcpyDeviceToHost, R.copy[s % 4]);
            if (e == cudaSuccess) e = cudaEventRecord(R.copy_ev[s], R.copy[s % 4]);
            if (e != cudaSuccess) {
                fail(s, cuda_fail(e, "resident copy"));
                continue;
            }
            R.state[s] = 1;
        }
        if (R.state[s] == 1) {
            const cudaError_t e = cudaEventQuery(R.copy_ev[s]);
            if (e == cudaErrorNotReady) continue;
            if (e == cudaSuccess) {
                out.push_back({R.req[s], VRT_OK, now_us(sv->t0), {}});
                R.state[s] = 2;
            } else {
                fail(s, cuda_fail(e, "resident copy"));
            }
        }
    }
    if (!R.live) return false;
    const cudaError_t e = cudaEventQuery(R.ended);
    if (e == cudaErrorNotReady) return false;
    R.live = false;
    R.closing = true;
    // every published view must be finished once the launch has ended
    for (uint32_t s = R.first_open; s < R.n_views; s++)
        if (R.state[s] == 0 && !resident_done_flag(R, s)) {
            if (e != cudaSuccess) cuda_fail(e, "resident launch");
            else set_error("resident launch ended before a published view finished");
            fail(s, VRT_ERR_DEVICE);
        }
    return true;
}

bool resident_idle(const Resident& R) {
    if (R.live) return false;
    for (uint32_t s = 0; s < R.n_views; s++)
        if (R.state[s] != 2) return false;
    return true;
}

// One pass of the resident scheduler over the queue, with sv->mu held by `lk`.  Returns
// true when it made progress and another pass may make more.
bool resident_schedule(vrt_server* sv, std::unique_lock<std::mutex>& lk) {
    Resident& R = sv->res;
    if (sv->queue.empty()) {
        if (sv->stop && R.live && !R.closing) resident_close(R);  // shutting down: no more work will come
        return false;
    }
    Request* front = sv->queue.front();
    if (front->kind == 1) {
        // an edit runs between frames: close the launch and wait for its end
        if (R.live) {
            if (!R.closing) resident_close(R);
            return false;
        }
        if (!resident_idle(R)) return false;
        sv->queue.pop_front();
        front->state = VRT_REQ_RUNNING;
        front->start_us = now_us(sv->t0);
        lk.unlock();
        vrt_status st = vrt_world_edit(sv->worlds[front->world], front->edits.data(),
                                       (uint32_t)front->edits.size(), sv->edit_stream);
        if (st == VRT_OK) st = vrt_world_wait(sv->worlds[front->world]);  // applied before later launches
        if (st == VRT_OK) st = refresh_world_table(sv);
        lk.lock();
        finish(sv, front, st, now_us(sv->t0));
        sv->done_cv.notify_all();
        return true;
    }
    const uint32_t mode = view_mode(front->view);
    // a launch that takes whole-path views is its own instantiation: a running one that
    // does not closes for the first such request, and the next launch takes every kind
    if (R.live && (R.closing || mode != R.mode || (view_full_path(front->view) && !R.full) || R.n_views >= R.cap)) {
        if (!R.closing) resident_close(R);  // a new launch takes the next requests
        return false;
    }
    if (!R.live && !resident_idle(R)) return false;  // the last launch's records are still copying
    std::vector<Request*> rs;
    const uint32_t room = R.live ? R.cap - R.n_views : R.cap;
    bool full = R.live && R.full;
    for (Request* r : sv->queue) {
        if (r->kind != 0 || view_mode(r->view) != mode || rs.size() >= sv->cfg.max_batch_requests ||
            rs.size() >= room || (R.live && view_full_path(r->view) && !R.full))
            break;
        full |= view_full_path(r->view);
        const uint32_t base = sv->pages.realloc(0, 0, r->pages);
        if (base == 0) break;  // budget full: wait for requests to finish
        r->page_base = base;
        rs.push_back(r);
    }
    if (rs.empty()) return false;
    const bool fresh = !R.live;
    vrt_status st = fresh ? resident_start(sv, mode, full) : VRT_OK;
    const bool ok = st == VRT_OK && resident_publish(sv, rs, st);
    if (ok && fresh) st = resident_launch(sv);
    if (ok && st == VRT_OK) {
        const double ts = now_us(sv->t0);
        for (Request* r : rs) {
            sv->queue.pop_front();
            r->state = VRT_REQ_RUNNING;
            r->start_us = ts;
            r->batch_size = (uint32_t)rs.size();
        }
        return true;
    }
    for (Request* r : rs) {  // not published: pages back, requests stay queued
        sv->pages.free(r->page_base, r->pages);
        r->page_base = 0;
    }
    if (st == VRT_OK) return false;  // the launch closed itself first: the next one takes them
    for (Request* r : rs) {          // a device or planning error fails these requests
        sv->queue.pop_front();
        finish(sv, r, st, now_us(sv->t0));
    }
    sv->done_cv.notify_all();
    return true;
}

// The scheduler thread of resident mode.  It polls the done flags and copy events
// without the server lock (a spinning thread that held it would starve submitters and
// waiters) and takes the lock only when a request finished, the launch ended, a
// submission or stop was signalled, or the last pass made progress.
void worker_resident(vrt_server* sv) {
    cudaSetDevice(sv->device);
    Resident& R = sv->res;
    uint64_t seen = ~0ull;
    bool again = true;
    std::vector<Finished> fin;
    for (;;) {
        const bool ended = resident_poll(sv, fin);
        const uint64_t sig = sv->signals.load(std::memory_order_acquire);
        if (again || ended || !fin.empty() || sig != seen) {
            seen = sig;
            std::unique_lock<std::mutex> lk(sv->mu);
            if (!fin.empty()) {
                for (Finished& f : fin) {
                    finish(sv, f.r, f.status, f.t);
                    if (f.status != VRT_OK) f.r->error = f.error;
                }
                fin.clear();
                sv->done_cv.notify_all();
            }
            if (sv->stop && sv->queue.empty() && resident_idle(R)) break;
            again = resident_schedule(sv, lk);
            if (again) continue;
        }
        // with work on the device, poll for finished views; otherwise sleep until signalled
        if (R.live || !resident_idle(R)) {
            std::this_thread::yield();
        } else {
            std::unique_lock<std::mutex> g(sv->sig_mu);
            sv->sig_cv.wait_for(g, std::chrono::milliseconds(1), [&] { return sv->signals.load() != seen; });
        }
    }
}

vrt_status resident_init(vrt_server* sv) {
    Resident& R = sv->res;
    int native = 0;
    VRT_CUDA(cudaDeviceGetAttribute(&native, cudaDevAttrHostNativeAtomicSupported, sv->device));
    if (!native) {
        set_error("resident serving needs host-native atomics between the device and host memory");
        return VRT_ERR_INVALID_ARG;
    }
    R.cap = kResidentViews;
    VRT_CUDA(cudaStreamCreateWithFlags(&R.stream, cudaStreamNonBlocking));
    VRT_CUDA(cudaStreamCreateWithFlags(&R.ctl, cudaStreamNonBlocking));
    for (cudaStream_t& c : R.copy) VRT_CUDA(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
    VRT_CUDA(cudaEventCreateWithFlags(&R.ended, cudaEventDisableTiming));
    VRT_CUDA(R.views.reserve((size_t)R.cap * sizeof(ViewDev)));
    VRT_CUDA(R.chunk_base.reserve((size_t)R.cap * sizeof(uint32_t)));
    VRT_CUDA(R.remaining.reserve((size_t)R.cap * sizeof(uint32_t)));
    VRT_CUDA(R.queue.reserve(256));
    void* mb = nullptr;
    VRT_CUDA(cudaHostAlloc(&mb, 64 + (size_t)R.cap * sizeof(uint32_t), cudaHostAllocMapped | cudaHostAllocPortable));
    std::memset(mb, 0, 64 + (size_t)R.cap * sizeof(uint32_t));
    R.mailbox = static_cast<unsigned long long*>(mb);
    R.done = reinterpret_cast<uint32_t*>(static_cast<uint8_t*>(mb) + 64);
    void* dmb = nullptr;
    VRT_CUDA(cudaHostGetDevicePointer(&dmb, mb, 0));
    R.d_mailbox = static_cast<unsigned long long*>(dmb);
    R.d_done = reinterpret_cast<uint32_t*>(static_cast<uint8_t*>(dmb) + 64);
    VRT_CUDA(cudaHostAlloc(&R.h_views, (size_t)R.cap * sizeof(ViewDev), cudaHostAllocDefault));
    VRT_CUDA(cudaHostAlloc(&R.h_cb, (size_t)R.cap * sizeof(uint32_t), cudaHostAllocDefault));
    VRT_CUDA(cudaHostAlloc(&R.h_rem, (size_t)R.cap * sizeof(uint32_t), cudaHostAllocDefault));
    VRT_CUDA(cudaHostAlloc(&R.h_hint, (2 * (size_t)R.cap + 1) * sizeof(unsigned long long), cudaHostAllocDefault));
    R.req.assign(R.cap, nullptr);
    R.state.assign(R.cap, 2);
    R.copy_ev.assign(R.cap, nullptr);
    for (auto& ev : R.copy_ev) VRT_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    return VRT_OK;
}

void resident_release(vrt_server* sv) {
    Resident& R = sv->res;
    if (R.stream) cudaStreamSynchronize(R.stream);
    for (cudaStream_t c : R.copy)
        if (c) cudaStreamSynchronize(c);
    for (cudaEvent_t ev : R.copy_ev)
        if (ev) cudaEventDestroy(ev);
    R.copy_ev.clear();
    if (R.ended) cudaEventDestroy(R.ended);
    for (cudaStream_t* s : {&R.stream, &R.ctl, &R.copy[0], &R.copy[1], &R.copy[2], &R.copy[3]})
        if (*s) cudaStreamDestroy(*s);
    R.views.release();
    R.chunk_base.release();
    R.remaining.release();
    R.queue.release();
    if (R.mailbox) cudaFreeHost(R.mailbox);
    if (R.h_views) cudaFreeHost(R.h_views);
    if (R.h_cb) cudaFreeHost(R.h_cb);
    if (R.h_rem) cudaFreeHost(R.h_rem);
    if (R.h_hint) cudaFreeHost(R.h_hint);
}

}  // namespace

extern "C" {

vrt_status vrt_host_alloc(size_t bytes, void** out) {
    if (!out) {
        set_error("null argument");
        return VRT_ERR_INVALID_ARG;
    }
    VRT_CUDA(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocPortable));
    return VRT_OK;
}

vrt_status vrt_host_free(void* p) {
    if (p) VRT_CUDA(cudaFreeHost(p));
    return VRT_OK;
}

vrt_status vrt_server_create(vrt_world* const* worlds, uint32_t n_worlds, const vrt_server_config* cfg_in,
                             vrt_server** out) {
    if (!out || !worlds || n_worlds == 0) {
        set_error("server needs worlds");
        return VRT_ERR_INVALID_ARG;
    }
    *out = nullptr;
    for (uint32_t i = 0; i < n_worlds; i++)
        if (!worlds[i] || worlds[i]->device != worlds[0]->device) {
            set_error("worlds must be non-null and on one device");
            return VRT_ERR_INVALID_ARG;
        }
    auto* sv = new vrt_server;
    sv->device = worlds[0]->device;
    sv->worlds.assign(worlds, worlds + n_worlds);
    sv->cfg = cfg_in ? *cfg_in : vrt_server_config{};
    if (sv->cfg.max_inflight == 0) sv->cfg.max_inflight = 2;
    if (sv->cfg.max_batch_requests == 0) sv->cfg.max_batch_requests = 256;
    auto fail = [&](vrt_status st) {
        vrt_server_destroy(sv, 0);
        return st;
    };
    vrt_status st = normalize_batch_config(&sv->cfg.batch, sv->bcfg);
    if (st != VRT_OK || sv->cfg.max_inflight > 16) {
        delete sv;
        if (st == VRT_OK) set_error("max_inflight must be <= 16");
        return st == VRT_OK ? VRT_ERR_INVALID_ARG : st;
    }
    DeviceScope ds;
    cudaError_t e = ds.enter(sv->device);
    if (e != cudaSuccess) return fail(cuda_fail(e, "set device"));
    if (sv->cfg.hbm_budget_bytes == 0) {
        size_t fr = 0, tot = 0;
        if ((e = cudaMemGetInfo(&fr, &tot)) != cudaSuccess) return fail(cuda_fail(e, "query free HBM"));
        sv->cfg.hbm_budget_bytes = fr / 4;
    }
    const uint64_t npages = std::max<uint64_t>(1, sv->cfg.hbm_budget_bytes / kPageBytes);
    if (npages > 0x3fffffffull) return fail((set_error("budget too large"), VRT_ERR_INVALID_ARG));
    if ((e = cudaMalloc(&sv->arena, npages * kPageBytes)) != cudaSuccess) return fail(cuda_fail(e, "output arena"));
    sv->pages.reset((uint32_t)npages);
    if ((e = cudaMalloc(&sv->d_worlds, sizeof(DevWorld) * n_worlds)) != cudaSuccess)
        return fail(cuda_fail(e, "world table"));
    if ((st = refresh_world_table(sv)) != VRT_OK) return fail(st);
    if ((e = cudaStreamCreateWithFlags(&sv->edit_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return fail(cuda_fail(e, "edit stream"));
    for (uint32_t i = 0; i < sv->cfg.max_inflight; i++) {
        auto s = std::make_unique<Slot>();
        s->server = sv;
        if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess)
            return fail(cuda_fail(e, "slot stream"));
        if ((e = cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming)) != cudaSuccess) {
            cudaStreamDestroy(s->stream);
            return fail(cuda_fail(e, "slot event"));
        }
        if ((e = s->queue.reserve(64)) != cudaSuccess) {
            cudaEventDestroy(s->done);
            cudaStreamDestroy(s->stream);
            return fail(cuda_fail(e, "slot queue"));
        }
        sv->slots.push_back(std::move(s));
    }
    const uint32_t modes = VRT_SERVE_RESIDENT | VRT_SERVE_LAUNCHES;
    if ((sv->cfg.flags & ~modes) || (sv->cfg.flags & modes) == modes)
        return fail((set_error("unknown server flags, or both modes asked for"), VRT_ERR_INVALID_ARG));
    if (sv->cfg.idle_us == 0) sv->cfg.idle_us = 500;
    bool resident = (sv->cfg.flags & VRT_SERVE_RESIDENT) != 0;
    if (!(sv->cfg.flags & modes)) {  // default: resident where the device supports it
        int native = 0;
        if ((e = cudaDeviceGetAttribute(&native, cudaDevAttrHostNativeAtomicSupported, sv->device)) != cudaSuccess)
            return fail(cuda_fail(e, "device attribute"));
        resident = native != 0;
    }
    sv->resident = resident;
    for (int m = 0; m < 3; m++)
        if ((st = persistent_grid(sv->device, sv->bcfg, false, m >= 1, m == 2, resident, false, sv->grid[m][0],
                                  sv->grid[m][1])) != VRT_OK)
            return fail(st);
    if (resident && (st = resident_init(sv)) != VRT_OK) return fail(st);
    sv->worker = resident ? std::thread(worker_resident, sv) : std::thread(worker_main, sv);
    *out = sv;
    return VRT_OK;
}

vrt_status vrt_server_destroy(vrt_server* sv, uint32_t timeout_ms) {
    if (!sv) return VRT_OK;
    vrt_status st = VRT_OK;
    if (sv->worker.joinable()) {
        st = vrt_server_drain(sv, timeout_ms);
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            sv->stop = true;
            // requests still queued after the wait are failed; launches in flight finish
            const double t = now_us(sv->t0);
            while (!sv->queue.empty()) {
                finish(sv, sv->queue.front(), VRT_ERR_QUEUE_TIMEOUT, t);
                sv->queue.pop_front();
            }
        }
        sv->signal();
        sv->worker.join();
    }
    DeviceScope ds;
    ds.enter(sv->device);
    for (auto& s : sv->slots) {
        if (s->stream) {
            cudaStreamSynchronize(s->stream);
            cudaStreamDestroy(s->stream);
        }
        if (s->done) cudaEventDestroy(s->done);
        s->views.release();
        s->chunk_base.release();
        s->queue.release();
        if (s->h_views) cudaFreeHost(s->h_views);
        if (s->h_cb) cudaFreeHost(s->h_cb);
    }
    resident_release(sv);
    if (sv->edit_stream) cudaStreamDestroy(sv->edit_stream);
    if (sv->arena) cudaFree(sv->arena);
    if (sv->d_worlds) cudaFree(sv->d_worlds);
    delete sv;
    return st;
}

vrt_status vrt_server_submit_render(vrt_server* sv, const vrt_view* view, vrt_hit* hits_host, uint64_t* ticket) {
    if (!sv || !view || !hits_host) {
        set_error("null argument");
        return VRT_ERR_INVALID_ARG;
    }
    vrt_status st = check_view(view);
    if (st != VRT_OK) return st;
    if (view->world >= sv->worlds.size()) {
        set_error("view references a world the server does not hold");
        return VRT_ERR_INVALID_ARG;
    }
    auto r = std::make_unique<Request>();
    r->kind = 0;
    r->view = *view;
    r->host_out = hits_host;
    r->records = view_record_count(*view);
    r->pages = (uint32_t)((r->records + kPageRecords - 1) / kPageRecords);
    r->submit_us = now_us(sv->t0);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stop) {
            set_error("server is stopping");
            return VRT_ERR_INVALID_ARG;
        }
        if (r->pages > sv->pages.capacity()) {
            sv->rejected++;
            set_error("request output exceeds the server's HBM budget");
            return VRT_ERR_OUT_OF_MEMORY;
        }
        r->id = sv->next_id++;
        if (ticket) *ticket = r->id;
        sv->queue.push_back(r.get());
        sv->reqs[r->id] = std::move(r);
        sv->outstanding++;
    }
    sv->signal();
    return VRT_OK;
}

vrt_status vrt_server_submit_edit(vrt_server* sv, uint32_t world, const vrt_edit* edits, uint32_t n,
                                  uint64_t* ticket) {
    if (!sv || (n && !edits) || world >= (sv ? sv->worlds.size() : 0)) {
        set_error("bad edit request");
        return VRT_ERR_INVALID_ARG;
    }
    auto r = std::make_unique<Request>();
    r->kind = 1;
    r->world = world;
    r->edits.assign(edits, edits + n);
    r->submit_us = now_us(sv->t0);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stop) {
            set_error("server is stopping");
            return VRT_ERR_INVALID_ARG;
        }
        r->id = sv->next_id++;
        if (ticket) *ticket = r->id;
        sv->queue.push_back(r.get());
        sv->reqs[r->id] = std::move(r);
        sv->outstanding++;
    }
    sv->signal();
    return VRT_OK;
}

vrt_status vrt_server_wait(vrt_server* sv, uint64_t ticket, uint32_t timeout_ms, vrt_request_info* info) {
    if (!sv) {
        set_error("null server");
        return VRT_ERR_INVALID_ARG;
    }
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) {
        set_error("unknown ticket");
        return VRT_ERR_NOT_FOUND;
    }
    Request* r = it->second.get();
    const bool ok = sv->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] {
        return r->state == VRT_REQ_DONE || r->state == VRT_REQ_FAILED;
    });
    if (info) {
        info->state = r->state;
        info->kind = r->kind;
        info->status = r->status;
        info->batch_size = r->batch_size;
        info->rays = r->records;
        info->submit_us = r->submit_us;
        info->start_us = r->start_us;
        info->done_us = r->done_us;
    }
    if (!ok) {
        set_error("request not finished within the timeout");
        return VRT_ERR_QUEUE_TIMEOUT;
    }
    if (r->state == VRT_REQ_FAILED) {
        set_error("request failed: " + r->error);
        return r->status;
    }
    return VRT_OK;
}

vrt_status vrt_server_drain(vrt_server* sv, uint32_t timeout_ms) {
    if (!sv) {
        set_error("null server");
        return VRT_ERR_INVALID_ARG;
    }
    std::unique_lock<std::mutex> lk(sv->mu);
    if (!sv->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return sv->outstanding == 0; })) {
        set_error("requests still outstanding after the timeout");
        return VRT_ERR_QUEUE_TIMEOUT;
    }
    return VRT_OK;
}

vrt_status vrt_server_get_stats(vrt_server* sv, int reset, vrt_server_stats* out) {
    if (!sv || !out) {
        set_error("null argument");
        return VRT_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lk(sv->mu);
    std::memset(out, 0, sizeof(*out));
    out->renders_done = sv->renders_done;
    out->edits_done = sv->edits_done;
    out->rejected = sv->rejected;
    out->launches = sv->launches;
    out->records = sv->records_done;
    out->resident = sv->resident ? 1u : 0u;
    double busy = sv->busy_total;
    if (sv->busy_since >= 0) busy += now_us(sv->t0) - sv->busy_since;
    out->busy_seconds = busy * 1e-6;
    if (!sv->lat.empty()) {
        std::vector<double> v = sv->lat;
        auto pct = [&](double q) {
            size_t k = (size_t)std::min<double>((double)v.size() - 1, std::floor(q * (double)(v.size() - 1) + 0.5));
            std::nth_element(v.begin(), v.begin() + (long)k, v.end());
            return v[k];
        };
        out->p50_us = pct(0.50);
        out->p99_us = pct(0.99);
        out->p999_us = pct(0.999);
        out->max_us = *std::max_element(v.begin(), v.end());
    }
    if (reset) {
        sv->lat.clear();
        sv->renders_done = sv->edits_done = sv->rejected = sv->launches = sv->records_done = 0;
        sv->busy_total = 0;
        if (sv->busy_since >= 0) sv->busy_since = now_us(sv->t0);
    }
    return VRT_OK;
}

}  // extern "C"
