// server.cu — continuous-batching SIFT service over resident engines.
//
// The serving form of the hot path: many detect_and_compute requests
// (src/sift.rs:1244-1355, SiftBackend::Cuda) of mixed resolutions in flight
// on one GPU at once.
//
//   slots      Each slot is a complete engine (engine.h) bound to one image
//              size: its pyramid, DoG, u8 and list arenas stay resident and
//              its CUDA graph for that size is captured once, together with
//              the engine's mapped pinned export buffer. A slot also owns a
//              completion event.
//   admission  A request waits in FIFO order until an idle slot of its size
//              exists, or a new slot fits the device-memory budget
//              (arena_bytes, counted as the slots' device bytes; a new slot
//              is admitted on its estimated footprint), or an idle slot of
//              another size can be evicted to make room; at most
//              max_inflight requests run at once.
//   service    One host thread owns every CUDA call of the server: it
//              launches admitted requests (H2D copy of the image, the slot's
//              graph — whose descriptor stage writes into the mapped host
//              buffer and whose last kernel (export.cu) writes the counters
//              and keypoints there — then an event) and polls the events of
//              running requests. A request
//              whose lists overflowed is re-run with grown lists; results stay
//              in the slot until the caller releases them.
//   overlap    Running requests are on different slots, hence different
//              streams: their kernels interleave on the device, and a request
//              that arrives while others run is launched at once if a slot is
//              free — continuous batching, not a queue in front of one engine.
//   autotune   Optionally, the first slot of each size times a few launch
//              shapes (fused blur radius limit, fused level tile height,
//              orientation and descriptor grids) by coordinate descent and
//              every slot of that size uses the fastest.
//
// sift_cuda_replay drives either this server or the plain one-call-per-image
// path with an open-loop request trace and reports per-request latency.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "engine.h"

namespace sift {
namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Device bytes an engine of size w x h holds after its first run (the arena
// layout of Engine::ensure_geometry and the initial list capacities of
// Engine::ensure_lists), used to admit a new slot before it exists.
uint64_t footprint_estimate(const SiftCudaParams& p, int storage, uint32_t w, uint32_t h) {
    const int O = (int)p.num_octaves, S = (int)p.num_intervals;
    const size_t es = storage == SIFT_CUDA_STORAGE_U8 ? 0 : (storage == SIFT_CUDA_STORAGE_F16 ? 2 : 4);
    uint64_t g = 0, u = 0, tmpb = 0, tmpo = 0, lt = 0, words = 0, caps = 0;
    uint32_t ow = w, oh = h;
    for (int o = 0; o < O; ++o) {
        const uint64_t pitch = align_up(std::max<uint32_t>(ow, 1), 32), plane = pitch * oh, nw = (ow + 31) / 32;
        g += plane * (S + 3) * es;
        u += plane * (S + 3);
        tmpb = std::max<uint64_t>(tmpb, plane);
        tmpo += align_up(plane, 256);
        if (o + 1 < O) lt = std::max<uint64_t>(lt, pitch * (oh / 2) * 4);
        const uint64_t wo = (uint64_t)S * oh * nw;
        words += wo * 4 * 2;
        caps += std::min<uint64_t>(std::max<uint64_t>(wo * 32 / 64, 1024), 1u << 28);
        ow /= 2;
        oh /= 2;
    }
    const uint64_t per_cand = 2 * sizeof(Keypoint) + kOriMaxPeaks * 4 + 3 * 4;
    const uint64_t per_out = sizeof(Keypoint) + kDescLen * 4;
    return align_up(std::max<uint32_t>(w, 1), 128) * h + g + u + tmpb + tmpo + lt + words + caps * per_cand +
           caps * per_out + (1u << 20);
}

}  // namespace

struct Request;

struct Slot {
    std::unique_ptr<Engine> eng;
    uint32_t w = 0, h = 0;
    uint64_t bytes = 0;  // device bytes of the engine
    cudaEvent_t done = nullptr;  // results are in the engine's mapped export buffer
    enum State { Idle, Running, Holding } state = Idle;
    Request* req = nullptr;
    uint64_t last_use = 0;
    int reruns = 0;

    ~Slot() {
        if (done) cudaEventDestroy(done);
    }
};

struct Request {
    uint64_t ticket = 0, tag = 0;
    uint32_t w = 0, h = 0, stride = 0;
    const uint8_t* img = nullptr;  // borrowed, or owned (pinned, from the pool)
    void* owned = nullptr;
    size_t owned_bytes = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    int status = 0;
    Slot* slot = nullptr;
};

struct TuneKey {
    uint32_t w, h;
    bool operator<(const TuneKey& o) const { return w != o.w ? w < o.w : h < o.h; }
};

struct Server {
    SiftCudaParams p{};
    SiftCudaServerOptions opt{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> pending;
    std::deque<Request*> finished;
    std::unordered_map<uint64_t, Request*> by_ticket;
    std::vector<std::unique_ptr<Slot>> slots;
    std::multimap<size_t, void*> pinned_free;  // owned-copy buffers
    std::map<TuneKey, Engine::Tuning> tuned;
    std::vector<std::pair<uint32_t, uint32_t>> creating;  // sizes of slots being created
    uint64_t next_ticket = 1, use_clock = 0, device_bytes = 0;
    uint32_t running = 0;
    bool stop = false;
    std::thread worker;
    // statistics
    uint64_t n_done = 0, n_reruns = 0, n_evicted = 0, max_pending = 0;

    ~Server() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv_work.notify_all();
        if (worker.joinable()) worker.join();
        cudaSetDevice(opt.device);
        for (auto& s : slots)
            if (s->eng) cudaStreamSynchronize(s->eng->st);
        for (auto& kv : by_ticket) release_request(kv.second);
        for (auto& kv : pinned_free) cudaFreeHost(kv.second);
        slots.clear();
    }

    void release_request(Request* r) {
        if (r->owned) pinned_free.emplace(r->owned_bytes, r->owned);
        delete r;
    }

    // -- slot management (service thread) ------------------------------------

    // Smaller images get more urgent streams: while a large image runs, the
    // block scheduler serves a small request's kernels first, so its latency
    // stays near its solo time. Tiers: up to 0.5 Mpx, up to 2.1 Mpx (1080p),
    // larger.
    int priority_for(uint32_t w, uint32_t h) const {
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return 0;
        const uint64_t area = (uint64_t)w * h;
        const int tier = area <= 500000 ? 0 : (area <= 2100000 ? 1 : 2);
        return std::min(least, greatest + tier);
    }

    // A new slot for w x h (service thread, lock NOT held: engine creation
    // allocates and captures).
    int make_slot(uint32_t w, uint32_t h, const Engine::Tuning* tune, std::unique_ptr<Slot>* out) {
        auto s = std::make_unique<Slot>();
        s->eng = std::make_unique<Engine>();
        s->eng->p = p;
        SiftCudaOptions eo;
        sift_cuda_options_default(&eo);
        eo.device = opt.device;
        eo.storage = opt.storage;
        s->eng->opt = eo;
        s->eng->priority = priority_for(w, h);
        if (int rc = s->eng->init()) return rc;
        if (int rc = s->eng->ensure_geometry(w, h)) return rc;
        CK(cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming), "cudaEventCreate");
        if (tune) s->eng->tune = *tune;
        s->w = w;
        s->h = h;
        s->bytes = s->eng->device_bytes();
        *out = std::move(s);
        return 0;
    }

    // Admission of r (lock held). Returns 0 and either *out (an idle slot of
    // r's size), or *create (a new slot of r's size fits: its estimated
    // footprint is reserved in device_bytes; idle slots of other sizes may
    // have been moved to *evicted to make room), or neither (r waits). A size
    // never holds more than max_inflight slots.
    int admit(Request* r, Slot** out, bool* create, std::vector<std::unique_ptr<Slot>>* evicted) {
        *out = nullptr;
        *create = false;
        uint32_t same = 0;
        for (auto& s : slots)
            if (s->w == r->w && s->h == r->h) {
                if (s->state == Slot::Idle) {
                    *out = s.get();
                    return 0;
                }
                ++same;
            }
        for (const auto& c : creating)
            if (c.first == r->w && c.second == r->h) ++same;
        if (same >= opt.max_inflight) return 0;
        const uint64_t need = footprint_estimate(p, opt.storage, r->w, r->h);
        if (need > opt.arena_bytes) return fail(SIFT_CUDA_ERR_CAPACITY, "image footprint above the arena budget");
        while (device_bytes + need > opt.arena_bytes) {
            size_t victim = slots.size();
            for (size_t i = 0; i < slots.size(); ++i) {
                const Slot* s = slots[i].get();
                if (s->state == Slot::Idle && (s->w != r->w || s->h != r->h) &&
                    (victim == slots.size() || s->last_use < slots[victim]->last_use))
                    victim = i;
            }
            if (victim == slots.size()) return 0;  // wait for running slots to finish
            device_bytes -= slots[victim]->bytes;
            evicted->push_back(std::move(slots[victim]));
            slots.erase(slots.begin() + (long)victim);
            ++n_evicted;
        }
        device_bytes += need;
        creating.emplace_back(r->w, r->h);
        *create = true;
        return 0;
    }

    // Times the slot's graph for a few launch shapes on the image already in
    // its engine, coordinate descent over the four knobs (service thread).
    int autotune(Slot* s) {
        Engine& e = *s->eng;
        cudaEvent_t a = nullptr, b = nullptr;
        CK(cudaEventCreate(&a), "cudaEventCreate");
        CK(cudaEventCreate(&b), "cudaEventCreate");
        // the graph timed is the one served: ending with the export
        if (int rc = e.ensure_export(e.last_n ? e.last_n : 4096)) return rc;
        auto time_cfg = [&](const Engine::Tuning& t, float* ms) -> int {
            e.tune = t;
            for (int k = 0; k < 2; ++k)
                if (int rc = e.run(true, true)) return rc;
            CK(cudaEventRecord(a, e.st), "event");
            for (int k = 0; k < 3; ++k)
                if (int rc = e.run(true, true)) return rc;
            CK(cudaEventRecord(b, e.st), "event");
            CK(cudaEventSynchronize(b), "event sync");
            CK(cudaEventElapsedTime(ms, a, b), "elapsed");
            return 0;
        };
        Engine::Tuning best = e.tune;
        float best_ms = 0.0f;
        int rc = time_cfg(best, &best_ms);
        // candidate values per knob: fused radius limit, level tile rows,
        // orientation CTAs/SM, descriptor CTAs/SM
        const int vals[4][3] = {{8, 4, 0}, {64, 32, 0}, {2, 4, 8}, {4, 8, 16}};
        const int nvals[4] = {3, 2, 3, 3};
        for (int knob = 0; knob < 4 && !rc; ++knob) {
            for (int v = 0; v < nvals[knob] && !rc; ++v) {
                Engine::Tuning t = best;
                if (knob == 0) t.fused_max_radius = vals[0][v];
                if (knob == 1) t.level_tile_rows = vals[1][v];
                if (knob == 2) t.ori_ctas_per_sm = vals[2][v];
                if (knob == 3) t.desc_ctas_per_sm = vals[3][v];
                if (t == best) continue;
                float ms = 0.0f;
                rc = time_cfg(t, &ms);
                if (!rc && ms < best_ms * 0.98f) {
                    best = t;
                    best_ms = ms;
                }
            }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        e.tune = best;
        std::lock_guard<std::mutex> g(mu);
        tuned[TuneKey{s->w, s->h}] = best;
        return rc;
    }

    int launch(Slot* s, Request* r) {
        Engine& e = *s->eng;
        if (int rc = e.upload(r->img, r->w, r->h, r->stride, cudaMemcpyHostToDevice)) return rc;
        bool tune = false;
        if (opt.autotune) {
            std::lock_guard<std::mutex> g(mu);
            tune = tuned.find(TuneKey{s->w, s->h}) == tuned.end();
        }
        if (tune)
            if (int rc = autotune(s)) return rc;
        return run_exported(s);
    }

    // One run of the slot's graph that ends with the export into the
    // engine's mapped buffer (descriptors written there by the descriptor
    // stage), then the completion event.
    int run_exported(Slot* s) {
        Engine& e = *s->eng;
        if (int rc = e.ensure_export(e.last_n ? e.last_n : 4096)) return rc;
        if (int rc = e.run(true, true)) return rc;
        CK(cudaEventRecord(s->done, e.st), "event record");
        return 0;
    }

    // A running slot whose event completed (lock held): re-run on overflow,
    // grow the export buffer when it was short, finish the request.
    // Returns 0 or a status; on 0 the slot is either running again or done.
    int complete(Slot* s) {
        Request* r = s->req;
        const Counters c = *s->eng->hx_ctr();
        bool retry = false;
        if (int rc = s->eng->grow_from(c, &retry)) return rc;
        if (retry) {
            ++n_reruns;
            return run_exported(s);
        }
        // more keypoints than the buffer held: grown, results moved (rare)
        if (int rc = s->eng->settle_export(c, true)) return rc;
        r->t_done = now_s();
        s->state = Slot::Holding;
        --running;
        finished.push_back(r);
        ++n_done;
        return 0;
    }

    void fail_request(Request* r, int rc) {
        r->status = rc ? rc : SIFT_CUDA_ERR_CUDA;
        r->t_done = now_s();
        if (r->slot && r->slot->state == Slot::Running) {
            r->slot->state = Slot::Holding;
            if (running) --running;
        }
        finished.push_back(r);
        ++n_done;
    }

    // The service loop. The lock guards the queues and the slot states only;
    // event polling, launches and slot creation or destruction run without
    // it, so submit, poll and release never wait behind CUDA calls.
    void service() {
        cudaSetDevice(opt.device);
        std::vector<Slot*> run_list, done_list;
        std::vector<cudaError_t> done_q;
        struct Start {
            Request* r;
            Slot* s;            // null: create a slot of r's size first
            uint64_t reserved;  // footprint reserved for that creation
        };
        std::vector<Start> starts;
        std::vector<std::unique_ptr<Slot>> evicted;
        std::unique_lock<std::mutex> lk(mu);
        while (true) {
            run_list.clear();
            for (auto& sp : slots)
                if (sp->state == Slot::Running && sp->req) run_list.push_back(sp.get());
            lk.unlock();
            done_list.clear();
            done_q.clear();
            for (Slot* s : run_list) {
                const cudaError_t q = cudaEventQuery(s->done);
                if (q == cudaErrorNotReady) continue;
                done_list.push_back(s);
                done_q.push_back(q);
            }
            lk.lock();
            bool progressed = !done_list.empty();
            for (size_t i = 0; i < done_list.size(); ++i) {
                Slot* s = done_list[i];
                const int rc = done_q[i] == cudaSuccess ? complete(s) : cuda_fail(done_q[i], "request");
                if (rc) fail_request(s->req, rc);
            }
            if (!finished.empty()) cv_done.notify_all();
            // admissions in FIFO order; a request that has to wait does not
            // hold back later requests of other sizes
            starts.clear();
            for (auto it = pending.begin(); it != pending.end() && running < opt.max_inflight;) {
                Request* r = *it;
                Slot* s = nullptr;
                bool create = false;
                const int rc = admit(r, &s, &create, &evicted);
                if (rc) {
                    it = pending.erase(it);
                    fail_request(r, rc);
                    progressed = true;
                    continue;
                }
                if (!s && !create) {
                    ++it;
                    continue;
                }
                it = pending.erase(it);
                if (s) {
                    s->state = Slot::Running;
                    s->req = nullptr;  // not polled until launched
                    s->last_use = ++use_clock;
                    r->slot = s;
                }
                r->t_start = now_s();
                ++running;
                progressed = true;
                starts.push_back(Start{r, s, create ? footprint_estimate(p, opt.storage, r->w, r->h) : 0});
            }
            if (stop) {
                // shutting down: requests not yet started fail
                while (!pending.empty()) {
                    Request* r = pending.front();
                    pending.pop_front();
                    r->status = SIFT_CUDA_ERR_INVALID_ARGUMENT;
                    r->t_done = now_s();
                    finished.push_back(r);
                }
            }
            if (!finished.empty()) cv_done.notify_all();
            if (stop && running == 0) break;
            lk.unlock();
            evicted.clear();  // engines of evicted slots are destroyed without the lock
            for (Start& st : starts) {
                Request* r = st.r;
                int rc = 0;
                if (!st.s) {
                    Engine::Tuning t{};
                    bool have_tune = false;
                    {
                        std::lock_guard<std::mutex> g(mu);
                        auto tt = tuned.find(TuneKey{r->w, r->h});
                        if (tt != tuned.end()) {
                            t = tt->second;
                            have_tune = true;
                        }
                    }
                    std::unique_ptr<Slot> fresh;
                    rc = make_slot(r->w, r->h, have_tune ? &t : nullptr, &fresh);
                    std::lock_guard<std::mutex> g(mu);
                    device_bytes -= st.reserved;
                    for (size_t k = 0; k < creating.size(); ++k)
                        if (creating[k].first == r->w && creating[k].second == r->h) {
                            creating.erase(creating.begin() + (long)k);
                            break;
                        }
                    if (!rc) {
                        Slot* s = fresh.get();
                        device_bytes += s->bytes;
                        s->state = Slot::Running;
                        s->last_use = ++use_clock;
                        r->slot = s;
                        slots.push_back(std::move(fresh));
                        st.s = s;
                    }
                }
                if (!rc) rc = launch(st.s, r);
                std::lock_guard<std::mutex> g(mu);
                if (rc) {
                    if (r->slot) r->slot->req = r;  // so that release frees the slot
                    else --running;
                    fail_request(r, rc);
                    cv_done.notify_all();
                } else {
                    st.s->req = r;  // now visible to the completion poll
                }
            }
            lk.lock();
            if (!progressed) {
                if (running == 0) {
                    cv_work.wait_for(lk, std::chrono::milliseconds(5));
                } else {
                    lk.unlock();
                    std::this_thread::sleep_for(std::chrono::microseconds(5));
                    lk.lock();
                }
            }
        }
    }
};

}  // namespace sift

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using sift::Server;

struct SiftCudaServer {
    Server s;
};

extern "C" {

void sift_cuda_server_options_default(SiftCudaServerOptions* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->device = 0;
    o->storage = SIFT_CUDA_STORAGE_U8;
    o->arena_bytes = 40ull << 30;
    o->max_inflight = 8;
    o->autotune = 0;
}

uint64_t sift_cuda_footprint_bytes(const SiftCudaParams* params, int32_t storage, uint32_t width, uint32_t height) {
    if (!params) return 0;
    return sift::footprint_estimate(*params, storage, width, height);
}

int sift_cuda_server_create(const SiftCudaParams* params, const SiftCudaServerOptions* opts, SiftCudaServer** out) {
    if (!out || !params) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "params or out is NULL");
    *out = nullptr;
    SiftCudaServerOptions o;
    sift_cuda_server_options_default(&o);
    if (opts) o = *opts;
    if (o.max_inflight == 0) o.max_inflight = 1;
    // validates params and the device like an engine would
    SiftCudaOptions eo;
    sift_cuda_options_default(&eo);
    eo.device = o.device;
    eo.storage = o.storage;
    SiftCudaEngine* probe = nullptr;
    if (int rc = sift_cuda_create(params, &eo, &probe)) return rc;
    sift_cuda_destroy(probe);
    auto* srv = new (std::nothrow) SiftCudaServer();
    if (!srv) return sift::fail(SIFT_CUDA_ERR_OUT_OF_MEMORY, "server allocation");
    srv->s.p = *params;
    srv->s.opt = o;
    srv->s.worker = std::thread([srv] { srv->s.service(); });
    *out = srv;
    return 0;
}

void sift_cuda_server_destroy(SiftCudaServer* server) { delete server; }

int sift_cuda_server_submit(SiftCudaServer* server, const uint8_t* img, uint32_t width, uint32_t height,
                            uint32_t stride, uint64_t tag, uint32_t flags, uint64_t* ticket) {
    sift::g_last_error.clear();
    if (!server || !ticket) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "server or ticket is NULL");
    if (!img || width == 0 || height == 0 || stride < width)
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "empty image, NULL pointer or stride < width");
    if (width > 65535u || height > 65535u) return sift::fail(SIFT_CUDA_ERR_UNSUPPORTED, "image sides above 65535");
    Server& S = server->s;
    auto* r = new (std::nothrow) sift::Request();
    if (!r) return sift::fail(SIFT_CUDA_ERR_OUT_OF_MEMORY, "request allocation");
    r->tag = tag;
    r->w = width;
    r->h = height;
    r->t_submit = sift::now_s();
    if (flags & SIFT_CUDA_SUBMIT_BORROW) {
        r->img = img;
        r->stride = stride;
    } else {
        const size_t bytes = (size_t)width * height;
        void* buf = nullptr;
        {
            std::lock_guard<std::mutex> lk(S.mu);
            auto it = S.pinned_free.lower_bound(bytes);
            if (it != S.pinned_free.end() && it->first <= 4 * bytes) {
                buf = it->second;
                r->owned_bytes = it->first;
                S.pinned_free.erase(it);
            }
        }
        if (!buf) {
            cudaSetDevice(S.opt.device);
            cudaError_t e = cudaHostAlloc(&buf, bytes, cudaHostAllocDefault);
            if (e != cudaSuccess) {
                delete r;
                return sift::cuda_fail(e, "cudaHostAlloc(request image)");
            }
            r->owned_bytes = bytes;
        }
        for (uint32_t y = 0; y < height; ++y)
            std::memcpy((uint8_t*)buf + (size_t)y * width, img + (size_t)y * stride, width);
        r->owned = buf;
        r->img = (const uint8_t*)buf;
        r->stride = width;
    }
    {
        std::lock_guard<std::mutex> lk(S.mu);
        r->ticket = S.next_ticket++;
        S.by_ticket[r->ticket] = r;
        S.pending.push_back(r);
        S.max_pending = std::max<uint64_t>(S.max_pending, S.pending.size());
        *ticket = r->ticket;
    }
    S.cv_work.notify_one();
    return 0;
}

int sift_cuda_server_poll(SiftCudaServer* server, SiftCudaServed* out, int64_t timeout_us) {
    if (!server || !out) return -SIFT_CUDA_ERR_INVALID_ARGUMENT;
    Server& S = server->s;
    std::unique_lock<std::mutex> lk(S.mu);
    if (S.finished.empty() && timeout_us != 0) {
        auto pred = [&] { return !S.finished.empty(); };
        if (timeout_us < 0)
            S.cv_done.wait(lk, pred);
        else
            S.cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), pred);
    }
    if (S.finished.empty()) return 0;
    sift::Request* r = S.finished.front();
    S.finished.pop_front();
    std::memset(out, 0, sizeof(*out));
    out->ticket = r->ticket;
    out->tag = r->tag;
    out->status = r->status;
    out->submit_s = r->t_submit;
    out->start_s = r->t_start;
    out->done_s = r->t_done;
    if (r->status == 0 && r->slot) {
        const sift::Engine& e = *r->slot->eng;
        out->n = e.hx_ctr()->n_oriented;
        out->kps = (const SiftCudaKeypoint*)e.hx_kps();
        out->desc = e.hx_desc();
    }
    return 1;
}

int sift_cuda_server_release(SiftCudaServer* server, uint64_t ticket) {
    if (!server) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "server is NULL");
    Server& S = server->s;
    {
        std::lock_guard<std::mutex> lk(S.mu);
        auto it = S.by_ticket.find(ticket);
        if (it == S.by_ticket.end()) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "unknown ticket");
        sift::Request* r = it->second;
        if (r->t_done == 0.0) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "request still running");
        if (r->slot && r->slot->req == r) {
            r->slot->state = sift::Slot::Idle;
            r->slot->req = nullptr;
        }
        S.by_ticket.erase(it);
        S.release_request(r);
    }
    S.cv_work.notify_one();
    return 0;
}

int sift_cuda_server_warm(SiftCudaServer* server, const uint8_t* img, uint32_t width, uint32_t height,
                          uint32_t stride, uint32_t count) {
    if (!server) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "server is NULL");
    std::vector<uint64_t> tickets;
    int rc = 0;
    for (uint32_t i = 0; i < count && !rc; ++i) {
        uint64_t t = 0;
        rc = sift_cuda_server_submit(server, img, width, height, stride, ~0ull, SIFT_CUDA_SUBMIT_BORROW, &t);
        if (!rc) tickets.push_back(t);
    }
    SiftCudaServed sv;
    for (size_t k = 0; k < tickets.size(); ++k) {
        if (sift_cuda_server_poll(server, &sv, -1) != 1) break;
        if (sv.status && !rc) rc = sift::fail(sv.status, "warm-up request failed");
        sift_cuda_server_release(server, sv.ticket);
    }
    return rc;
}

int sift_cuda_server_stats(SiftCudaServer* server, SiftCudaServerStats* out) {
    if (!server || !out) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "server or out is NULL");
    Server& S = server->s;
    std::lock_guard<std::mutex> lk(S.mu);
    std::memset(out, 0, sizeof(*out));
    out->slots = (uint32_t)S.slots.size();
    out->running = S.running;
    out->pending = (uint32_t)S.pending.size();
    out->device_bytes = S.device_bytes;
    out->completed = S.n_done;
    out->reruns = S.n_reruns;
    out->evicted = S.n_evicted;
    out->max_pending = S.max_pending;
    return 0;
}

int sift_cuda_server_tuning(SiftCudaServer* server, uint32_t width, uint32_t height, int32_t* knobs3) {
    if (!server || !knobs3) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "server or knobs is NULL");
    Server& S = server->s;
    std::lock_guard<std::mutex> lk(S.mu);
    auto it = S.tuned.find(sift::TuneKey{width, height});
    sift::Engine::Tuning t{};
    if (it != S.tuned.end()) t = it->second;
    knobs3[0] = t.fused_max_radius;
    knobs3[1] = t.ori_ctas_per_sm;
    knobs3[2] = t.desc_ctas_per_sm;
    return it != S.tuned.end() ? 1 : 0;
}

int sift_cuda_server_tuning_knobs(SiftCudaServer* server, uint32_t width, uint32_t height, int32_t* knobs,
                                  uint32_t n_knobs) {
    if (!server || (!knobs && n_knobs)) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "server or knobs is NULL");
    Server& S = server->s;
    std::lock_guard<std::mutex> lk(S.mu);
    auto it = S.tuned.find(sift::TuneKey{width, height});
    sift::Engine::Tuning t{};
    if (it != S.tuned.end()) t = it->second;
    const int32_t all[4] = {t.fused_max_radius, t.level_tile_rows, t.ori_ctas_per_sm, t.desc_ctas_per_sm};
    for (uint32_t i = 0; i < n_knobs && i < 4; ++i) knobs[i] = all[i];
    return it != S.tuned.end() ? 1 : 0;
}

// Open-loop replay: request i is due at t0 + reqs[i].arrival_s; latency is
// measured from that due time to the moment its result is in host memory.
int sift_cuda_replay(SiftCudaServer* server, const SiftCudaParams* params, const SiftCudaOptions* opts,
                     const SiftCudaReplayImage* images, uint32_t n_images, const SiftCudaReplayRequest* reqs,
                     uint32_t n_reqs, SiftCudaReplayResult* results, double* wall_s) {
    sift::g_last_error.clear();
    if (!images || !reqs || !results || (!server && !params))
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "NULL argument");
    for (uint32_t i = 0; i < n_reqs; ++i)
        if (reqs[i].image >= n_images) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "image index out of range");
    if (!server) {
        // the plain path: one synchronous detect_and_compute per request, an
        // engine per image size (so no request pays a re-layout)
        std::map<sift::TuneKey, SiftCudaEngine*> engines;
        int rc = 0;
        for (uint32_t i = 0; i < n_images && !rc; ++i) {
            const auto& im = images[i];
            sift::TuneKey k{im.width, im.height};
            if (engines.count(k)) continue;
            SiftCudaEngine* e = nullptr;
            rc = sift_cuda_create(params, opts, &e);
            if (rc) break;
            engines[k] = e;
            SiftCudaResult res;
            rc = sift_cuda_detect_and_compute_view(e, im.data, im.width, im.height, im.stride, &res);
        }
        const double t0 = sift::now_s();
        for (uint32_t i = 0; i < n_reqs && !rc; ++i) {
            const double due = t0 + reqs[i].arrival_s;
            while (sift::now_s() < due) {
            }
            const auto& im = images[reqs[i].image];
            SiftCudaResult res;
            const int st = sift_cuda_detect_and_compute_view(engines[sift::TuneKey{im.width, im.height}], im.data,
                                                             im.width, im.height, im.stride, &res);
            results[i].latency_s = sift::now_s() - due;
            results[i].n = st ? 0 : res.n;
            results[i].status = st;
        }
        if (wall_s) *wall_s = sift::now_s() - t0;
        for (auto& kv : engines) sift_cuda_destroy(kv.second);
        return rc;
    }
    Server& S = server->s;
    std::atomic<uint32_t> got{0};
    std::vector<double> due(n_reqs, 0.0);
    double t0 = 0.0;
    std::thread consumer([&] {
        SiftCudaServed sv;
        while (got.load() < n_reqs) {
            if (sift_cuda_server_poll(server, &sv, 100000) != 1) continue;
            const uint32_t i = (uint32_t)sv.tag;
            results[i].latency_s = sv.done_s - due[i];
            results[i].n = sv.n;
            results[i].status = sv.status;
            sift_cuda_server_release(server, sv.ticket);
            got.fetch_add(1);
        }
    });
    t0 = sift::now_s();
    int rc = 0;
    uint32_t submitted = 0;
    for (uint32_t i = 0; i < n_reqs; ++i) {
        due[i] = t0 + reqs[i].arrival_s;
        while (sift::now_s() < due[i]) {
        }
        const auto& im = images[reqs[i].image];
        uint64_t ticket = 0;
        rc = sift_cuda_server_submit(server, im.data, im.width, im.height, im.stride, i, SIFT_CUDA_SUBMIT_BORROW,
                                     &ticket);
        if (rc) break;
        ++submitted;
    }
    if (rc) {
        // count the requests that never went in as done so the consumer ends
        for (uint32_t i = submitted; i < n_reqs; ++i) results[i].status = rc;
        got.fetch_add(n_reqs - submitted);
    }
    consumer.join();
    if (wall_s) *wall_s = sift::now_s() - t0;
    (void)S;
    return rc;
}

}  // extern "C"
