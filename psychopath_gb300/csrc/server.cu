// Render server (psy_server_* / psy_submit / psy_poll / psy_wait / psy_cancel
// of include/psy_gpu.h): a scheduling thread that keeps several scenes
// resident, admits requests by HBM budget and packs the rows of concurrent
// requests of a scene into shared wavefronts.
//
// The reference has no request loop: one process renders one scene,
// bucket by bucket, on CPU threads (Renderer::render, src/renderer.rs:76-191).
// What is kept from it is the unit of independent work -- a path per
// (pixel, sample index, seed) whose result does not depend on what else is
// in flight (src/renderer.rs:241-310) -- which is what lets requests share
// wavefront queues without changing their images.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/psy_gpu.h"
#include "kernels.cuh"
#include "scene_handle.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kRing = 4;  // wave descriptor slots per lane (>= waves in flight)

struct Req {
    uint64_t id = 0;
    PsyRequest r{};
    uint64_t rows_left_samples() const { return (uint64_t)(r.height - next_row) * r.width * r.spp; }
    uint32_t state = PSY_REQ_QUEUED;
    int err = 0;
    float *d_img = nullptr;   // where accumulate writes (own buffer or the caller's)
    bool own_img = false;
    uint64_t img_bytes = 0;   // budget charge (own buffer only)
    uint32_t next_row = 0;    // first row not yet put in a wave
    uint32_t outstanding = 0; // segments in waves not yet finished
    bool cancel = false;
    bool overflow = false;
    uint32_t waves = 0, shared_waves = 0;
    Clock::time_point t_submit, t_admit, t_done;
};

// A finished request whose result the finisher copies out (copy: to the
// caller's host buffer) before it is published.
struct Finish {
    Req *q;
    bool copy;
};

struct Flight {
    cudaEvent_t ev = nullptr;
    int slot = 0;
    std::vector<Req *> reqs;  // one entry per segment
};

struct Lane {
    PsyScene *scene = nullptr;
    cudaStream_t st = nullptr;
    WaveBufs B{};
    std::vector<void *> allocs;
    uint64_t bytes = 0;
    WaveDesc *h_ring = nullptr;  // pinned staging of the descriptors
    int *h_err = nullptr;        // pinned error word of each slot's wave
    cudaEvent_t ev[kRing] = {};
    std::deque<Flight> inflight;
    std::deque<Req *> active;    // admitted requests with rows left, in arrival order
    WaveGraph graphs[kRing];
    int next_slot = 0;
};

}  // namespace

struct PsyServer {
    PsyServerOptions opt{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work;   // wakes the scheduler
    std::condition_variable cv_done;   // wakes psy_wait
    std::thread thr;
    bool stop = false;
    int fatal = 0;
    std::string fatal_msg;
    std::vector<std::unique_ptr<Lane>> lanes;
    std::map<uint64_t, std::unique_ptr<Req>> reqs;
    std::deque<Req *> pending;
    uint64_t next_id = 1;
    uint32_t n_active = 0;
    uint64_t used = 0, peak = 0;
    uint64_t done = 0, samples_done = 0, waves = 0, launches = 0;
    cudaMemPool_t pool = nullptr;
    cudaStream_t copy_st = nullptr;
    // finished requests whose results the finisher thread copies out, so
    // the scheduler keeps issuing waves meanwhile (a copy to pageable host
    // memory blocks the calling thread)
    std::thread fin_thr;
    std::condition_variable cv_fin;
    std::deque<std::vector<Finish>> fin_q;
    bool fin_stop = false;
};

namespace {

int fail(int code, const std::string &m) { return psy_fail(code, m); }

double secs(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

void fill_status(const Req &q, PsyRequestStatus *st) {
    std::memset(st, 0, sizeof(*st));
    st->state = q.state;
    st->error = q.err;
    st->samples = (uint64_t)q.r.width * q.r.height * q.r.spp;
    auto now = Clock::now();
    bool admitted = q.state != PSY_REQ_QUEUED && q.t_admit != Clock::time_point{};
    st->queued_s = secs(q.t_submit, admitted ? q.t_admit : now);
    bool finished = q.state == PSY_REQ_DONE || q.state == PSY_REQ_CANCELLED || q.state == PSY_REQ_FAILED;
    st->latency_s = secs(q.t_submit, finished ? q.t_done : now);
    st->waves = q.waves;
    st->shared_waves = q.shared_waves;
}

bool finished(const Req &q) {
    return q.state == PSY_REQ_DONE || q.state == PSY_REQ_CANCELLED || q.state == PSY_REQ_FAILED;
}

// Called with the lock held: marks the server failed and every unfinished
// request FAILED.
void set_fatal(PsyServer *s, int code, const std::string &msg) {
    if (!s->fatal) {
        s->fatal = code;
        s->fatal_msg = msg;
    }
    auto now = Clock::now();
    for (auto &kv : s->reqs) {
        Req &q = *kv.second;
        if (!finished(q)) {
            q.state = PSY_REQ_FAILED;
            q.err = code;
            q.t_done = now;
        }
    }
    s->pending.clear();
    for (auto &l : s->lanes) l->active.clear();
    s->cv_done.notify_all();
}

std::string cuda_msg(cudaError_t e, const char *what) { return std::string(what) + ": " + cudaGetErrorString(e); }

// Scheduling order (PsyServerOptions.policy): under PSY_SCHED_SHORTEST,
// requests older than aging_ms first (in arrival order), then the others by
// fewest samples left, ties in arrival order; under FIFO, arrival order.
// `samples` gives a request's remaining work.
template <class Work>
void sched_order(const PsyServer *s, std::vector<Req *> &v, Work samples) {
    if (s->opt.policy != PSY_SCHED_SHORTEST) return;  // v is in arrival order already
    auto now = Clock::now();
    double age_s = s->opt.aging_ms * 1e-3;
    std::stable_sort(v.begin(), v.end(), [&](const Req *a, const Req *b) {
        bool oa = secs(a->t_submit, now) > age_s, ob = secs(b->t_submit, now) > age_s;
        if (oa != ob) return oa;
        if (oa) return false;  // both aged: arrival order (stable)
        return samples(a) < samples(b);
    });
}

// Packs rows of the lane's active requests into the next wave and issues it.
// Called with the lock held.  Returns false when there was nothing to issue.
bool issue_wave(PsyServer *s, Lane &L, std::string &err) {
    const uint32_t cap = L.B.cap;
    int slot = L.next_slot;
    WaveDesc &d = L.h_ring[slot];
    std::memset(&d, 0, sizeof(d));
    Flight f;
    f.slot = slot;
    uint32_t paths = 0, pix = 0;
    std::vector<Req *> order(L.active.begin(), L.active.end());
    sched_order(s, order, [](const Req *q) { return q->rows_left_samples(); });
    for (Req *q : order) {
        if (d.nseg >= PSY_WAVE_MAX_SEGS || paths >= cap) break;
        if (q->cancel) continue;
        uint32_t row_paths = q->r.width * q->r.spp;
        uint32_t fit = (cap - paths) / row_paths;
        if (fit == 0) break;  // keep the order: this request waits for the next wave
        uint32_t take = std::min(fit, q->r.height - q->next_row);
        WaveSeg &g = d.seg[d.nseg++];
        g.x0 = 0; g.y0 = q->next_row; g.w = q->r.width; g.h = take;
        g.spp = q->r.spp; g.seed = q->r.seed;
        g.img_w = q->r.width; g.img_h = q->r.height;
        g.out = q->d_img; g.out_stride = q->r.width;
        g.ystep = 1; g.orow0 = q->next_row;
        g.path_begin = paths; g.pix_begin = pix;
        paths += take * row_paths;
        pix += take * q->r.width;
        q->next_row += take;
        q->outstanding++;
        f.reqs.push_back(q);
    }
    // drop fully scheduled requests from the active list (cancelled ones are
    // taken out by the scheduler, which also finishes them)
    for (auto it = L.active.begin(); it != L.active.end();) {
        if ((*it)->next_row >= (*it)->r.height) it = L.active.erase(it);
        else ++it;
    }
    if (d.nseg == 0) return false;
    d.npaths = paths;
    d.npix = pix;
    for (size_t i = 0; i < f.reqs.size(); i++) {
        Req *q = f.reqs[i];
        bool first = std::find(f.reqs.begin(), f.reqs.begin() + i, q) == f.reqs.begin() + i;
        if (first) {
            q->waves++;
            bool other = false;
            for (Req *o : f.reqs) other |= (o != q);
            if (other) q->shared_waves++;
        }
    }
    WaveDesc *d_slot = L.B.waves + slot;
    PsyScene *sc = L.scene;
    cudaError_t e = cudaMemcpyAsync(d_slot, &d, sizeof(WaveDesc), cudaMemcpyHostToDevice, L.st);
    if (e == cudaSuccess) e = cudaMemsetAsync(L.B.err, 0, sizeof(int), L.st);
    if (e != cudaSuccess) {
        err = cuda_msg(e, "wave descriptor upload");
        return false;
    }
    int r = s->opt.use_graphs ? launch_wave_graph(sc, L.B, L.graphs[slot], d_slot, cap, cap, L.st)
                              : launch_wave(sc, L.B, d_slot, cap, cap, L.st, nullptr, nullptr);
    if (r != PSY_OK) {
        err = "wave launch failed";
        return false;
    }
    e = cudaMemcpyAsync(&L.h_err[slot], L.B.err, sizeof(int), cudaMemcpyDeviceToHost, L.st);
    if (e == cudaSuccess) e = cudaEventRecord(L.ev[slot], L.st);
    if (e != cudaSuccess) {
        err = cuda_msg(e, "wave completion record");
        return false;
    }
    f.ev = L.ev[slot];
    L.inflight.push_back(std::move(f));
    L.next_slot = (slot + 1) % kRing;
    s->waves++;
    // camera + (trace, shadow-result shade, hit shade) per iteration +
    // accumulate, and the queue-ordering kernels between iterations when
    // the lane orders its queues (keys + scan + scatter, or keys + three
    // kernels per 8-bit radix pass)
    uint64_t iters = 2 * sc->g.max_bounces + 3;
    int bits = (sc->sort_bits > 0 && L.B.stage) ? sc->sort_bits : 0;
    uint64_t per_binning = bits == 0 ? 0 : (bits <= 16 ? 3 : 1 + 3 * (uint64_t)((bits + 7) / 8));
    s->launches += 2 + iters * 3 + per_binning * (iters - 1);
    return true;
}


void scheduler(PsyServer *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        if (s->stop) break;
        std::vector<Finish> fin;
        std::string err;
        // 1. completed waves
        for (auto &lp : s->lanes) {
            Lane &L = *lp;
            while (!L.inflight.empty()) {
                cudaError_t q = cudaEventQuery(L.inflight.front().ev);
                if (q == cudaErrorNotReady) break;
                if (q != cudaSuccess) {
                    err = cuda_msg(q, "wave execution");
                    break;
                }
                Flight f = std::move(L.inflight.front());
                L.inflight.pop_front();
                bool ovf = L.h_err[f.slot] != 0;
                for (Req *r : f.reqs) {
                    r->outstanding--;
                    if (ovf) r->overflow = true;
                }
                for (Req *r : f.reqs) {
                    if (r->outstanding == 0 && !finished(*r) &&
                        (r->cancel || r->next_row >= r->r.height)) {
                        r->state = PSY_REQ_RUNNING;  // stays running until the copy is done
                        r->outstanding = ~0u;        // marks "finishing" (no second finish)
                        fin.push_back({r, !r->cancel && r->own_img && r->r.xyz_out != nullptr});
                    }
                }
            }
            if (!err.empty()) break;
            // cancelled requests leave the active list; those with no wave
            // in flight finish now
            for (auto it = L.active.begin(); it != L.active.end();) {
                Req *r = *it;
                if (!r->cancel) {
                    ++it;
                    continue;
                }
                it = L.active.erase(it);
                if (r->outstanding == 0) {
                    r->outstanding = ~0u;
                    fin.push_back({r, false});
                }
            }
        }
        if (!err.empty()) {
            set_fatal(s, PSY_E_CUDA, err);
            break;
        }
        // 2. finish: the finisher thread copies the results out and
        // publishes them; the scheduler goes on issuing waves
        if (!fin.empty()) {
            s->fin_q.push_back(std::move(fin));
            s->cv_fin.notify_one();
        }
        // 3. admission, in policy order, while the budget and the active
        // limit allow (a request that does not fit the budget waits, and so
        // do the ones after it)
        std::vector<Req *> cand;
        for (Req *q : s->pending) {
            if (q->cancel) {
                q->state = PSY_REQ_CANCELLED;
                q->t_done = Clock::now();
                s->cv_done.notify_all();
            } else {
                cand.push_back(q);
            }
        }
        if (cand.size() != s->pending.size()) s->pending.assign(cand.begin(), cand.end());
        sched_order(s, cand, [](const Req *q) { return (uint64_t)q->r.width * q->r.height * q->r.spp; });
        for (Req *q : cand) {
            if (s->n_active >= s->opt.max_active) break;
            uint64_t bytes = q->r.d_xyz_out ? 0 : (uint64_t)q->r.width * q->r.height * 12;
            if (s->used + bytes > s->opt.hbm_budget_bytes) break;
            Lane &L = *s->lanes[q->r.scene];
            if (bytes) {
                void *p = nullptr;
                cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, s->pool, L.st);
                if (e != cudaSuccess) {
                    set_fatal(s, psy_cuda_fail(e, "request image"), cuda_msg(e, "request image"));
                    break;
                }
                q->d_img = static_cast<float *>(p);
                q->own_img = true;
            } else {
                q->d_img = q->r.d_xyz_out;
            }
            q->img_bytes = bytes;
            s->used += bytes;
            s->peak = std::max(s->peak, s->used);
            s->n_active++;
            q->state = PSY_REQ_RUNNING;
            q->t_admit = Clock::now();
            s->pending.erase(std::find(s->pending.begin(), s->pending.end(), q));
            L.active.push_back(q);
        }
        if (s->fatal) break;
        // 4. issue waves while lanes have room
        bool any_inflight = false;
        for (auto &lp : s->lanes) {
            Lane &L = *lp;
            while ((int)L.inflight.size() < (int)s->opt.waves_in_flight && !L.active.empty()) {
                if (!issue_wave(s, L, err)) break;
            }
            if (!err.empty()) break;
            any_inflight |= !L.inflight.empty();
        }
        if (!err.empty()) {
            set_fatal(s, PSY_E_CUDA, err);
            break;
        }
        // 5. wait: poll the GPU while waves are in flight; with requests
        // waiting for memory or a slot, sleep until the finisher (or a
        // submit or cancel) wakes the loop, at most 1 ms; else until work
        if (any_inflight)
            s->cv_work.wait_for(lk, std::chrono::microseconds(100));
        else if (!s->pending.empty())
            s->cv_work.wait_for(lk, std::chrono::milliseconds(1));
        else
            s->cv_work.wait(lk, [s] { return s->stop || !s->pending.empty(); });
    }
}

// The finisher thread: copies finished requests' results to the callers'
// host buffers and frees their images (lock released), then publishes the
// requests' final states and wakes the scheduler (memory freed for
// admission) and the waiters.
void finisher(PsyServer *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv_fin.wait(lk, [s] { return s->fin_stop || !s->fin_q.empty(); });
        if (s->fin_q.empty()) break;  // stopping with nothing left
        std::vector<Finish> fin = std::move(s->fin_q.front());
        s->fin_q.pop_front();
        lk.unlock();
        cudaError_t ce = cudaSuccess;
        for (Finish &f : fin) {
            if (f.copy && ce == cudaSuccess)
                ce = cudaMemcpyAsync(f.q->r.xyz_out, f.q->d_img, (size_t)f.q->r.width * f.q->r.height * 12,
                                     cudaMemcpyDeviceToHost, s->copy_st);
        }
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(s->copy_st);
        for (Finish &f : fin)
            if (f.q->own_img && ce == cudaSuccess) ce = cudaFreeAsync(f.q->d_img, s->copy_st);
        lk.lock();
        if (ce != cudaSuccess) {
            set_fatal(s, PSY_E_CUDA, cuda_msg(ce, "result copy"));
            s->cv_work.notify_all();
            continue;
        }
        auto now = Clock::now();
        for (Finish &f : fin) {
            Req &q = *f.q;
            q.outstanding = 0;
            q.d_img = q.own_img ? nullptr : q.d_img;
            s->used -= q.img_bytes;
            s->n_active--;
            q.t_done = now;
            if (q.cancel) {
                q.state = PSY_REQ_CANCELLED;
            } else if (q.overflow) {
                q.state = PSY_REQ_FAILED;
                q.err = PSY_E_OVERFLOW;
            } else {
                q.state = PSY_REQ_DONE;
                s->samples_done += (uint64_t)q.r.width * q.r.height * q.r.spp;
            }
            s->done++;
        }
        s->cv_done.notify_all();
        s->cv_work.notify_one();
    }
}

}  // namespace

extern "C" {

int psy_server_create(const PsyServerOptions *opts, PsyServer **out) {
    if (!out) return fail(PSY_E_INVALID, "out is null");
    *out = nullptr;
    auto s = std::make_unique<PsyServer>();
    if (opts) s->opt = *opts;
    if (s->opt.hbm_budget_bytes == 0) s->opt.hbm_budget_bytes = 120ull * 1000 * 1000 * 1000;
    if (s->opt.wave_paths == 0) s->opt.wave_paths = 1u << 22;
    if (s->opt.wave_paths < 1024) return fail(PSY_E_INVALID, "wave_paths below 1024");
    if (s->opt.max_active == 0) s->opt.max_active = 64;
    if (s->opt.waves_in_flight == 0) s->opt.waves_in_flight = 2;
    if (s->opt.waves_in_flight > kRing) return fail(PSY_E_INVALID, "waves_in_flight above 4");
    if (s->opt.policy > PSY_SCHED_SHORTEST) return fail(PSY_E_INVALID, "unknown scheduling policy");
    if (s->opt.aging_ms == 0) s->opt.aging_ms = 1000;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) return psy_cuda_fail(e, "cudaGetDevice");
    cudaMemPoolProps pp{};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = s->device;
    e = cudaMemPoolCreate(&s->pool, &pp);
    if (e != cudaSuccess) return psy_cuda_fail(e, "cudaMemPoolCreate");
    uint64_t keep = ~0ull;  // keep freed request images reserved for the next ones
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    e = cudaStreamCreateWithFlags(&s->copy_st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaMemPoolDestroy(s->pool);
        return psy_cuda_fail(e, "copy stream");
    }
    PsyServer *raw = s.release();
    raw->thr = std::thread(scheduler, raw);
    raw->fin_thr = std::thread(finisher, raw);
    *out = raw;
    return PSY_OK;
}

int psy_server_add_scene(PsyServer *s, PsyScene *scene, uint32_t *lane) {
    if (!s || !scene || !lane) return fail(PSY_E_INVALID, "null argument");
    auto L = std::make_unique<Lane>();
    L->scene = scene;
    uint64_t need = scene->device_bytes;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->fatal) return fail(s->fatal, s->fatal_msg);
    }
    // queue-ordering scratch when the scene orders its wavefront queues
    // (its tuned launch), so served waves run the scene's own configuration
    int r = alloc_wave_bufs(L->B, s->opt.wave_paths, kRing, scene->sort_bits > 0, L->allocs, L->bytes);
    auto cleanup = [&]() {
        for (void *p : L->allocs) cudaFree(p);
        if (L->h_ring) cudaFreeHost(L->h_ring);
        if (L->h_err) cudaFreeHost(L->h_err);
        for (auto &ev : L->ev)
            if (ev) cudaEventDestroy(ev);
        if (L->st) cudaStreamDestroy(L->st);
    };
    cudaError_t e = cudaSuccess;
    if (r == PSY_OK) e = cudaHostAlloc((void **)&L->h_ring, kRing * sizeof(WaveDesc), cudaHostAllocDefault);
    if (r == PSY_OK && e == cudaSuccess) e = cudaHostAlloc((void **)&L->h_err, kRing * sizeof(int), cudaHostAllocDefault);
    if (r == PSY_OK && e == cudaSuccess) e = cudaStreamCreateWithFlags(&L->st, cudaStreamNonBlocking);
    for (int i = 0; i < kRing && r == PSY_OK && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&L->ev[i], cudaEventDisableTiming);
    if (r == PSY_OK && e != cudaSuccess) r = psy_cuda_fail(e, "lane setup");
    if (r != PSY_OK) {
        cleanup();
        return r;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    need += L->bytes;
    if (s->used + need > s->opt.hbm_budget_bytes) {
        cleanup();
        return fail(PSY_E_NOMEM, "scene and lane buffers exceed the server's HBM budget");
    }
    s->used += need;
    s->peak = std::max(s->peak, s->used);
    *lane = (uint32_t)s->lanes.size();
    s->lanes.push_back(std::move(L));
    return PSY_OK;
}

int psy_submit(PsyServer *s, const PsyRequest *req, uint64_t *id) {
    if (!s || !req || !id) return fail(PSY_E_INVALID, "null argument");
    if (req->width == 0 || req->height == 0 || req->spp == 0) return fail(PSY_E_INVALID, "empty request");
    if (!req->xyz_out && !req->d_xyz_out) return fail(PSY_E_INVALID, "request has no output buffer");
    if ((uint64_t)req->width * req->spp > s->opt.wave_paths)
        return fail(PSY_E_INVALID, "one row of the request (width * spp paths) exceeds the wave size");
    auto q = std::make_unique<Req>();
    q->r = *req;
    q->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->fatal) return fail(s->fatal, s->fatal_msg);
    if (req->scene >= s->lanes.size()) return fail(PSY_E_INVALID, "unknown scene lane");
    uint64_t bytes = req->d_xyz_out ? 0 : (uint64_t)req->width * req->height * 12;
    uint64_t fixed = 0;
    for (auto &l : s->lanes) fixed += l->bytes + l->scene->device_bytes;
    if (fixed + bytes > s->opt.hbm_budget_bytes)
        return fail(PSY_E_NOMEM, "request image can never fit the server's HBM budget");
    q->id = s->next_id++;
    *id = q->id;
    s->pending.push_back(q.get());
    s->reqs.emplace(q->id, std::move(q));
    s->cv_work.notify_one();
    return PSY_OK;
}

int psy_poll(PsyServer *s, uint64_t id, PsyRequestStatus *st) {
    if (!s || !st) return fail(PSY_E_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(PSY_E_NOTFOUND, "unknown request id");
    fill_status(*it->second, st);
    return PSY_OK;
}

int psy_wait(PsyServer *s, uint64_t id, double timeout_s, PsyRequestStatus *st) {
    if (!s) return fail(PSY_E_INVALID, "null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(PSY_E_NOTFOUND, "unknown request id");
    Req *q = it->second.get();
    timeout_s = std::min(std::max(timeout_s, 0.0), 1e6);
    auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
    bool ok = s->cv_done.wait_until(lk, deadline, [q] { return finished(*q); });
    if (st) fill_status(*q, st);
    if (!ok) return fail(PSY_E_TIMEOUT, "request not finished before the timeout");
    return PSY_OK;
}

int psy_cancel(PsyServer *s, uint64_t id) {
    if (!s) return fail(PSY_E_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(PSY_E_NOTFOUND, "unknown request id");
    Req &q = *it->second;
    if (finished(q)) return fail(PSY_E_INVALID, "request already finished");
    q.cancel = true;
    s->cv_work.notify_one();
    return PSY_OK;
}

int psy_server_stats(PsyServer *s, PsyServerStats *st) {
    if (!s || !st) return fail(PSY_E_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(st, 0, sizeof(*st));
    st->requests_done = s->done;
    st->samples_done = s->samples_done;
    st->waves = s->waves;
    st->kernel_launches = s->launches;
    st->hbm_used_bytes = s->used;
    st->hbm_peak_bytes = s->peak;
    st->hbm_budget_bytes = s->opt.hbm_budget_bytes;
    st->queued = (uint32_t)s->pending.size();
    st->active = s->n_active;
    return PSY_OK;
}

int psy_server_destroy(PsyServer *s) {
    if (!s) return PSY_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->thr.joinable()) s->thr.join();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->fin_stop = true;  // the finisher completes the batches handed to it, then leaves
        s->cv_fin.notify_all();
    }
    if (s->fin_thr.joinable()) s->fin_thr.join();
    for (auto &lp : s->lanes) cudaStreamSynchronize(lp->st);
    cudaStreamSynchronize(s->copy_st);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto now = Clock::now();
        for (auto &kv : s->reqs) {
            Req &q = *kv.second;
            if (q.own_img && q.d_img) cudaFree(q.d_img);
            q.d_img = nullptr;
            if (!finished(q)) {
                q.state = PSY_REQ_CANCELLED;
                q.t_done = now;
            }
        }
        s->cv_done.notify_all();
    }
    for (auto &lp : s->lanes) {
        Lane &L = *lp;
        for (auto &g : L.graphs) g.reset();
        for (void *p : L.allocs) cudaFree(p);
        if (L.h_ring) cudaFreeHost(L.h_ring);
        if (L.h_err) cudaFreeHost(L.h_err);
        for (auto &ev : L.ev)
            if (ev) cudaEventDestroy(ev);
        if (L.st) cudaStreamDestroy(L.st);
    }
    if (s->copy_st) cudaStreamDestroy(s->copy_st);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return PSY_OK;
}

}  // extern "C"
