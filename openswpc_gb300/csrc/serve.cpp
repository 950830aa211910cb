// Serving form: a request loop with continuous batching over the C ABI.
//
// Request life cycle (swpc_serve_* in include/swpc_gpu.h):
//
//   submit -> QUEUED -> a loader thread runs the host set-up (swpc_host_load:
//   medium, sources, stations; no device) -> WAITING: the request holds its
//   loader until the admitted simulations leave room for it inside the HBM
//   budget (strict arrival order) -> the loader creates the simulation on the
//   device and uploads it (swpc_host_materialize) -> the scheduler adds it to
//   the running batch at the next quantum boundary -> RUNNING -> when its nt
//   steps are done the scheduler copies its receiver traces to host memory,
//   frees its device memory and returns the bytes to the budget -> DONE.
//
// The scheduler thread owns the batch: per quantum it launches `quantum`
// steps of every running simulation as one fused launch sequence
// (swpc_batch_run), waits, retires finished members and rebuilds the batch
// when membership changed.  Host set-up of arriving requests runs on the
// loader threads meanwhile, so it overlaps the device work.  The reference
// runs one simulation per process and has no counterpart.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "../../include/swpc_gpu.h"

namespace swpc {
int set_err(int code, const std::string& msg);
}

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    long long id = 0;
    std::string path;
    int state = SWPC_REQ_QUEUED;
    long long ticket = -1;  // admission order
    double t[4] = {-1, -1, -1, -1};
    long long bytes = 0;
    swpc_sim* sim = nullptr;
    int nt = 0, done = 0;
    double points = 0;
    std::map<int, std::vector<float>> wav;  // kind -> (nst, ncmp, ntw)
    int nst = 0, ntw = 0;
    std::string msg;  // error message of a failed request
};

int ncmp(int kind) { return (kind == SWPC_WAV_V || kind == SWPC_WAV_U) ? 3 : 6; }

}  // namespace

struct swpc_server {
    swpc_serve_config cfg{};
    int device = 0;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_load, cv_admit, cv_sched, cv_done;
    bool stop = false;
    long long next_id = 1, next_ticket = 0, admit_next = 0;
    std::set<long long> skip;  // tickets that left the admission line early
    std::deque<Req*> incoming;
    std::vector<Req*> ready, active;
    std::map<long long, std::unique_ptr<Req>> reqs;
    double granted = 0, peak = 0;
    long long n_done = 0, n_failed = 0, quanta = 0, rebuilds = 0;
    double updates = 0;
    std::vector<std::thread> loaders;
    std::thread scheduler;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    // caller holds mu
    void advance_line() {
        while (skip.count(admit_next)) {
            skip.erase(admit_next);
            ++admit_next;
        }
    }
    // caller holds mu; the failing call ran on this thread, whose last error
    // message is kept with the request
    void fail(Req* r, int rc) {
        char buf[512];
        swpc_gpu_last_error(buf, sizeof buf);
        r->msg = buf;
        r->state = rc < 0 ? rc : SWPC_E_CUDA;
        r->t[3] = now();
        ++n_failed;
        cv_done.notify_all();
    }

    void loader_main() {
        cudaSetDevice(device);
        for (;;) {
            Req* r;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_load.wait(lk, [&] { return stop || !incoming.empty(); });
                if (stop) return;
                r = incoming.front();
                incoming.pop_front();
                r->state = SWPC_REQ_LOADING;
                r->ticket = next_ticket++;
            }
            swpc_request* h = nullptr;
            int rc = swpc_host_load(r->path.c_str(), &h);
            swpc_dims d{};
            long long bytes = 0;
            if (rc == 0) {
                swpc_host_request_dims(h, &d);
                bytes = swpc_host_request_bytes(h);
                if (bytes < 0) rc = (int)bytes;
            }
            {
                std::unique_lock<std::mutex> lk(mu);
                if (rc == 0 && (double)bytes > cfg.hbm_budget)
                    rc = swpc::set_err(SWPC_E_NOMEM, "request " + r->path + " needs more device memory than the serving budget");
                if (rc) {
                    skip.insert(r->ticket);
                    advance_line();
                    cv_admit.notify_all();
                    fail(r, rc);
                    lk.unlock();
                    swpc_host_request_free(h);
                    continue;
                }
                r->state = SWPC_REQ_WAITING;
                r->bytes = bytes;
                r->nt = d.nt;
                r->points = (double)d.nx * d.ny * d.nz;
                cv_admit.wait(lk, [&] {
                    return stop || (admit_next == r->ticket && granted + (double)bytes <= cfg.hbm_budget &&
                                    (int)(active.size() + ready.size()) < cfg.max_active);
                });
                if (stop) {
                    lk.unlock();
                    swpc_host_request_free(h);
                    return;
                }
                ++admit_next;
                advance_line();
                granted += (double)bytes;
                peak = std::max(peak, granted);
                r->t[1] = now();
                cv_admit.notify_all();
            }
            swpc_sim* sim = nullptr;
            rc = swpc_host_materialize(h, &sim);
            swpc_host_request_free(h);
            std::lock_guard<std::mutex> lk(mu);
            if (rc) {
                granted -= (double)r->bytes;
                cv_admit.notify_all();
                fail(r, rc);
                continue;
            }
            r->sim = sim;
            ready.push_back(r);
            cv_sched.notify_all();
        }
    }

    // Copy the traces of a finished member to host memory, free its device
    // memory and hand its bytes back.  Called by the scheduler without mu.
    void retire(Req* r, int status) {
        if (status == 0) {
            int nst = 0, ntw = 0;
            swpc_gpu_query(r->sim, &ntw, &nst, nullptr, nullptr, nullptr);
            for (int kind : {SWPC_WAV_V, SWPC_WAV_U, SWPC_WAV_STRESS, SWPC_WAV_STRAIN}) {
                std::vector<float> w((size_t)nst * ncmp(kind) * ntw);
                if (w.empty()) continue;
                if (swpc_gpu_fetch_waveforms(r->sim, kind, w.data()) == 0) r->wav[kind] = std::move(w);
            }
            r->nst = nst;
            r->ntw = ntw;
            if (cfg.write_sac) {
                status = swpc_host_write_sac(r->sim, nullptr);
                if (!status) status = swpc_host_write_snp(r->sim, nullptr);
                if (!status) status = swpc_host_write_green(r->sim, nullptr);
            }
        }
        swpc_gpu_destroy(r->sim);
        r->sim = nullptr;
        std::lock_guard<std::mutex> lk(mu);
        granted -= (double)r->bytes;
        if (status == 0) {
            r->state = SWPC_REQ_DONE;
            r->t[3] = now();
            ++n_done;
            cv_done.notify_all();
        } else {
            fail(r, status);
        }
        cv_admit.notify_all();
    }

    void scheduler_main() {
        cudaSetDevice(device);
        swpc_batch* batch = nullptr;
        bool rebuild = false;
        for (;;) {
            std::vector<Req*> joined;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_sched.wait(lk, [&] { return stop || !ready.empty() || !active.empty(); });
                if (stop) break;
                joined.swap(ready);
                for (Req* r : joined) {
                    r->state = SWPC_REQ_RUNNING;
                    r->t[2] = now();
                    active.push_back(r);
                }
            }
            if (!joined.empty()) rebuild = true;
            if (rebuild) {
                if (batch) swpc_batch_destroy(batch);
                batch = nullptr;
                std::vector<swpc_sim*> sims;
                for (Req* r : active) sims.push_back(r->sim);
                int rc = swpc_batch_create(sims.data(), (int)sims.size(), &batch);
                {
                    std::lock_guard<std::mutex> lk(mu);
                    ++rebuilds;
                }
                if (rc) {
                    std::vector<Req*> all;
                    {
                        std::lock_guard<std::mutex> lk(mu);
                        all.swap(active);
                    }
                    for (Req* r : all) retire(r, rc);
                    continue;
                }
                rebuild = false;
            }
            int k = cfg.quantum;
            for (Req* r : active) k = std::min(k, r->nt - r->done);
            int rc = k > 0 ? swpc_batch_run(batch, k) : 0;
            cudaStreamSynchronize((cudaStream_t)swpc_batch_stream(batch));
            double pts = 0;
            std::vector<std::pair<Req*, int>> out;
            std::vector<Req*> keep;
            for (Req* r : active) {
                r->done += k;
                pts += r->points * k;
                int st = rc ? rc : swpc_gpu_sync(r->sim);
                if (st || r->done >= r->nt) out.emplace_back(r, st);
                else keep.push_back(r);
            }
            {
                std::lock_guard<std::mutex> lk(mu);
                active.swap(keep);
                ++quanta;
                updates += pts;
            }
            for (auto& q : out) retire(q.first, q.second);
            if (!out.empty()) rebuild = true;
        }
        if (batch) swpc_batch_destroy(batch);
    }
};

extern "C" {

int swpc_serve_create(const swpc_serve_config* cfg, swpc_server** out) {
    if (!out) return swpc::set_err(SWPC_E_ARG, "null argument to swpc_serve_create");
    *out = nullptr;
    auto* s = new swpc_server();
    if (cfg) s->cfg = *cfg;
    if (s->cfg.max_active <= 0) s->cfg.max_active = 128;
    if (s->cfg.quantum <= 0) s->cfg.quantum = 50;
    if (s->cfg.prep_threads <= 0) s->cfg.prep_threads = 4;
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        delete s;
        return swpc::set_err(SWPC_E_CUDA, "no CUDA device for the server");
    }
    if (s->cfg.hbm_budget <= 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            delete s;
            return swpc::set_err(SWPC_E_CUDA, "cudaMemGetInfo failed");
        }
        s->cfg.hbm_budget = 0.8 * (double)fr;
    }
    s->t0 = Clock::now();
    for (int q = 0; q < s->cfg.prep_threads; ++q) s->loaders.emplace_back([s] { s->loader_main(); });
    s->scheduler = std::thread([s] { s->scheduler_main(); });
    *out = s;
    return 0;
}

int swpc_serve_submit(swpc_server* s, const char* inf_path, long long* id) {
    if (!s || !inf_path) return swpc::set_err(SWPC_E_ARG, "null argument to swpc_serve_submit");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return swpc::set_err(SWPC_E_STATE, "server is shutting down");
    auto r = std::make_unique<Req>();
    r->id = s->next_id++;
    r->path = inf_path;
    r->t[0] = s->now();
    s->incoming.push_back(r.get());
    if (id) *id = r->id;
    s->reqs[r->id] = std::move(r);
    s->cv_load.notify_one();
    return 0;
}

int swpc_serve_state(swpc_server* s, long long id) {
    if (!s) return swpc::set_err(SWPC_E_ARG, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return swpc::set_err(SWPC_E_ARG, "unknown request id");
    return it->second->state;
}

int swpc_serve_wait(swpc_server* s, long long id, double timeout_s) {
    if (!s) return swpc::set_err(SWPC_E_ARG, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return swpc::set_err(SWPC_E_ARG, "unknown request id");
    Req* r = it->second.get();
    auto fin = [&] { return r->state == SWPC_REQ_DONE || r->state < 0; };
    if (timeout_s < 0) s->cv_done.wait(lk, fin);
    else s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), fin);
    return r->state;
}

int swpc_serve_result(swpc_server* s, long long id, int kind, float* buf, size_t n_floats, int* nst, int* ntw) {
    if (!s) return swpc::set_err(SWPC_E_ARG, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return swpc::set_err(SWPC_E_ARG, "unknown request id");
    Req* r = it->second.get();
    if (r->state != SWPC_REQ_DONE) return swpc::set_err(SWPC_E_STATE, "request is not finished");
    auto w = r->wav.find(kind);
    if (w == r->wav.end()) return swpc::set_err(SWPC_E_STATE, "the request recorded no traces of this kind");
    if (nst) *nst = r->nst;
    if (ntw) *ntw = r->ntw;
    if (!buf) return 0;
    if (n_floats < w->second.size()) return swpc::set_err(SWPC_E_ARG, "result buffer too small");
    std::memcpy(buf, w->second.data(), w->second.size() * sizeof(float));
    return 0;
}

int swpc_serve_error(swpc_server* s, long long id, char* buf, size_t n) {
    if (!s) return swpc::set_err(SWPC_E_ARG, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return swpc::set_err(SWPC_E_ARG, "unknown request id");
    const std::string& m = it->second->msg;
    if (buf && n) {
        size_t k = std::min(n - 1, m.size());
        std::memcpy(buf, m.data(), k);
        buf[k] = 0;
    }
    return (int)m.size();
}

int swpc_serve_times(swpc_server* s, long long id, double* t4) {
    if (!s || !t4) return swpc::set_err(SWPC_E_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return swpc::set_err(SWPC_E_ARG, "unknown request id");
    for (int q = 0; q < 4; ++q) t4[q] = it->second->t[q];
    return 0;
}

int swpc_serve_release(swpc_server* s, long long id) {
    if (!s) return swpc::set_err(SWPC_E_ARG, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return swpc::set_err(SWPC_E_ARG, "unknown request id");
    if (it->second->state != SWPC_REQ_DONE && it->second->state >= 0)
        return swpc::set_err(SWPC_E_STATE, "request is still in flight");
    s->reqs.erase(it);
    return 0;
}

int swpc_serve_drain(swpc_server* s) {
    if (!s) return swpc::set_err(SWPC_E_ARG, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] {
        for (auto& kv : s->reqs)
            if (kv.second->state != SWPC_REQ_DONE && kv.second->state >= 0) return false;
        return true;
    });
    return 0;
}

int swpc_serve_stats(swpc_server* s, double* st) {
    if (!s || !st) return swpc::set_err(SWPC_E_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    double waiting = 0;
    for (auto& kv : s->reqs)
        if (kv.second->state == SWPC_REQ_LOADING || kv.second->state == SWPC_REQ_WAITING) waiting += 1;
    st[0] = (double)s->n_done;
    st[1] = (double)s->n_failed;
    st[2] = (double)(s->active.size() + s->ready.size());
    st[3] = waiting;
    st[4] = (double)s->incoming.size();
    st[5] = s->granted;
    st[6] = s->peak;
    st[7] = (double)s->quanta;
    st[8] = (double)s->rebuilds;
    st[9] = s->updates;
    return 0;
}

int swpc_serve_destroy(swpc_server* s) {
    if (!s) return 0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_load.notify_all();
    s->cv_admit.notify_all();
    s->cv_sched.notify_all();
    for (auto& t : s->loaders) t.join();
    if (s->scheduler.joinable()) s->scheduler.join();
    // simulations still on the device (admitted but unfinished) are freed
    for (Req* r : s->active) if (r->sim) swpc_gpu_destroy(r->sim);
    for (Req* r : s->ready) if (r->sim) swpc_gpu_destroy(r->sim);
    delete s;
    return 0;
}

}  // extern "C"
