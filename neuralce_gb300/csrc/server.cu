// Job server of libnce_gb300 (serving form): admission by a device-memory budget, continuous batching of CE
// jobs into persistent batch launches on a few lanes, NeuralCE jobs chunk by chunk on side streams, all state resident on the
// device while a job runs.  Host code only; the device work is the engines' own entry points.
//
// Threads: the caller's threads only touch host structures under `mu` (submit, poll, cancel, query never wait
// for the device).  The io thread admits jobs (upload, initial energies or caches) and retires them (outputs
// copied to the caller's host buffers, device memory returned with cudaFreeAsync) on its own stream, so neither
// stalls the device work; the CE thread keeps eight lanes (streams) of persistent batch launches busy with the
// running CE jobs (up to max_batch jobs per launch; a job joins the next launch as soon as its previous one has
// completed), the NeuralCE thread each running NeuralCE job's next chunk as soon as its previous one has completed
// (jobs spread over `nce_streams` streams, jobs of one model on one stream).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace nce {
namespace {

struct SJob {
    int64_t id = 0;
    nce_job_desc d{};                 // output pointers as given; input pointers replaced by the host copies
    int64_t N = 0;
    int32_t n_cols = 0, mo = 0, binary = 0, C0 = 0, D = 0, depth = 0, lf = 0;   // lf: runs the local-field kernel
    std::vector<int8_t> sig; std::vector<float> beta; std::vector<int32_t> lid;
    const int8_t *sig_src = nullptr;  // the initial occupancies: `sig`, or the caller's buffer (NCE_JOB_BORROW_SIGMA)
    int64_t bytes = 0;
    int status = NCE_JOB_QUEUED, error = 0;
    std::string msg;
    int64_t done = 0;
    bool cancel = false;
    double t_submit = -1.0, t_start = -1.0, t_end = -1.0;
    char *dev = nullptr;              // one device block holding the job's state
    nce_pt_state st{};
    nce_nce_state nst{};
    int32_t chunks = 0, anchor = 1;
    bool inflight = false;            // part of a launch that has not completed (its worker thread only)
    int64_t pending_steps = 0;        // NeuralCE: steps of the chunk in flight
    cudaEvent_t ev = nullptr;         // NeuralCE: completion of the job's chunk in flight
    ~SJob() { if (ev) cudaEventDestroy(ev); }
    cudaStream_t stream = nullptr;
};

inline int64_t al256(int64_t x) { return (x + 255) / 256 * 256; }

// device bytes of a job's state, and the offsets of its arrays
struct Plan {
    std::vector<int64_t> off;
    int64_t total = 0;
    int64_t add(int64_t n) { off.push_back(total); total += al256(std::max<int64_t>(n, 1)); return off.back(); }
};

Plan ce_plan(int32_t R, int64_t N, int32_t n_cols, bool track, bool lf) {
    Plan p;
    p.add((int64_t)R * N);                       // 0 sigma
    p.add(8ll * R);                              // 1 E
    p.add(4ll * R);                              // 2 beta
    p.add(4ll * R); p.add(4ll * R); p.add(4ll * R);   // 3 ros, 4 sor, 5 lid
    p.add(8ll * R);                              // 6 E_min
    p.add(8ll * R);                              // 7 n_acc
    p.add(8);                                    // 8 n_ex
    p.add(track ? 8ll * R * n_cols : 0);         // 9 cv
    p.add(lf ? 8ll * R * N : 0);                 // 10 local fields
    return p;
}

Plan nce_plan(int32_t R, int64_t N, int32_t C0, int32_t D, int32_t depth) {
    Plan p;
    p.add((int64_t)R * N);                       // 0 sigma
    p.add(4ll * R * N * C0);                     // 1 h0
    p.add(depth >= 2 ? 4ll * (depth - 1) * R * N * D : 0);   // 2 hmid
    p.add(4ll * R * N);                          // 3 e
    p.add(8ll * R);                              // 4 E
    p.add(4ll * R);                              // 5 beta
    p.add(4ll * R); p.add(4ll * R); p.add(4ll * R);   // 6 ros, 7 sor, 8 lid
    p.add(8ll * R);                              // 9 n_acc
    p.add(8);                                    // 10 n_ex
    return p;
}

}  // namespace
}  // namespace nce

using namespace nce;

struct nce_server {
    nce_server_config cfg{};
    int device = 0;
    std::mutex mu;
    std::condition_variable wake;
    std::map<int64_t, std::shared_ptr<SJob>> jobs;
    std::deque<std::shared_ptr<SJob>> pending[2];
    std::vector<std::shared_ptr<SJob>> active[2];
    std::deque<std::shared_ptr<SJob>> retiring[2];   // finished or cancelled running jobs, for the io threads
    int64_t next_id = 1, bytes_used = 0;
    int64_t n_done = 0, n_cancelled = 0, n_failed = 0, rounds[2] = {0, 0};
    std::atomic<int64_t> attempts{0};
    std::atomic<bool> stop{false};
    std::thread worker[4];                           // CE launches, NeuralCE chunks, CE io, NeuralCE io
    std::chrono::steady_clock::time_point t0;
    cudaStream_t io_streams[2] = {nullptr, nullptr};
    std::vector<cudaStream_t> ce_streams, nce_streams;
    int rr = 0;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

// retire a job whose device memory is released (called with mu held)
void release_locked(nce_server *S, SJob &j, int status) {
    if (j.dev) S->bytes_used -= j.bytes;
    j.dev = nullptr;
    j.status = status;
    j.t_end = S->now();
    if (status == NCE_JOB_DONE) ++S->n_done;
    else if (status == NCE_JOB_CANCELLED) ++S->n_cancelled;
    else if (status == NCE_JOB_FAILED) ++S->n_failed;
}

// pick the pending jobs of `kind` that fit the budget now (mu held); reserves their bytes
std::vector<std::shared_ptr<SJob>> admit_locked(nce_server *S, int kind) {
    std::vector<std::shared_ptr<SJob>> out;
    const double t = S->now();
    // the oldest pending job of either kind; nothing overtakes it once it has waited starve_s
    std::shared_ptr<SJob> oldest;
    for (int k = 0; k < 2; ++k)
        for (auto &p : S->pending[k])
            if (!p->cancel && (!oldest || p->id < oldest->id)) oldest = p;
    auto &q = S->pending[kind];
    for (auto it = q.begin(); it != q.end();) {
        auto &p = *it;
        if (p->cancel) {
            release_locked(S, *p, NCE_JOB_CANCELLED);
            it = q.erase(it);
            continue;
        }
        if (oldest && oldest != p && t - oldest->t_submit > S->cfg.starve_s && oldest->id < p->id) break;
        if (S->bytes_used + p->bytes <= S->cfg.hbm_budget) {
            S->bytes_used += p->bytes;
            p->dev = reinterpret_cast<char *>(1);      // reserved; allocated by the worker
            p->status = NCE_JOB_RUNNING;
            p->t_start = t;
            out.push_back(p);
            it = q.erase(it);
        } else {
            ++it;
        }
    }
    return out;
}

void fail_job(nce_server *S, SJob &j, int rc) {
    std::lock_guard<std::mutex> lk(S->mu);
    j.error = rc;
    j.msg = last_error();
    if (j.dev) S->bytes_used -= j.bytes;
    j.dev = nullptr;
    j.status = NCE_JOB_FAILED;
    j.t_end = S->now();
    ++S->n_failed;
}

int start_ce(nce_server *S, SJob &j, cudaStream_t s) {
    const int32_t R = j.d.R;
    const bool track = j.binary != 0;
    Plan p = ce_plan(R, j.N, j.n_cols, track, j.lf != 0);
    void *base = nullptr;
    NCE_CUDA(cudaMallocAsync(&base, (size_t)p.total, s));
    j.dev = (char *)base;
    char *b = j.dev;
    nce_pt_state &st = j.st;
    std::memset(&st, 0, sizeof(st));
    st.R = R; st.N = j.N; st.sigma = (int8_t *)(b + p.off[0]); st.E = (double *)(b + p.off[1]); st.beta_slot = (float *)(b + p.off[2]);
    st.rep_of_slot = (int32_t *)(b + p.off[3]); st.slot_of_rep = (int32_t *)(b + p.off[4]); st.ladder_id = (int32_t *)(b + p.off[5]);
    st.E_min_rep = (double *)(b + p.off[6]); st.n_acc = (int64_t *)(b + p.off[7]); st.n_ex = (int64_t *)(b + p.off[8]);
    st.cv = track ? (int64_t *)(b + p.off[9]) : nullptr;
    std::vector<int32_t> iota(R);
    for (int i = 0; i < R; ++i) iota[i] = i;
    std::vector<double> inf(R, std::numeric_limits<double>::infinity());
    NCE_CUDA(cudaMemcpyAsync(st.sigma, j.sig_src, (size_t)R * j.N, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync((void *)st.beta_slot, j.beta.data(), 4 * (size_t)R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync((void *)st.ladder_id, j.lid.data(), 4 * (size_t)R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.rep_of_slot, iota.data(), 4 * (size_t)R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.slot_of_rep, iota.data(), 4 * (size_t)R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.E_min_rep, inf.data(), 8 * (size_t)R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemsetAsync(st.n_acc, 0, 8 * (size_t)R, s));
    NCE_CUDA(cudaMemsetAsync(st.n_ex, 0, 8, s));
    nce_ce_handle h = (nce_ce_handle)j.d.model;
    // one pass over the configurations: the exact sums, and the float64 energies from them
    int rc = track ? nce_ce_cluster_counts(h, st.sigma, R, st.cv, s) : nce_ce_energy(h, st.sigma, R, 64, st.E, s);
    if (rc) return rc;
    if (track) { rc = nce_ce_energy_from_counts(h, st.cv, R, st.E, s); if (rc) return rc; }
    if (j.lf) {
        st.field = (int64_t *)(b + p.off[10]);
        rc = nce_ce_field_init(h, st.sigma, R, st.field, s);
        if (rc) return rc;
    }
    NCE_CUDA(cudaMemcpyAsync(st.E_min_rep, st.E, 8, cudaMemcpyDeviceToDevice, s));   // replica 0, as PT set-up does
    return NCE_OK;                 // the io thread synchronises once for all the jobs it admits in one pass
}

int start_nce(nce_server *S, SJob &j, cudaStream_t s) {
    const int32_t R = j.d.R;
    Plan p = nce_plan(R, j.N, j.C0, j.D, j.depth);
    void *base = nullptr;
    NCE_CUDA(cudaMallocAsync(&base, (size_t)p.total, s));
    j.dev = (char *)base;
    char *b = j.dev;
    nce_nce_state &st = j.nst;
    std::memset(&st, 0, sizeof(st));
    st.R = R; st.N = j.N; st.sigma = (int8_t *)(b + p.off[0]); st.h0 = (float *)(b + p.off[1]);
    st.hmid = j.depth >= 2 ? (float *)(b + p.off[2]) : nullptr; st.e = (float *)(b + p.off[3]); st.E = (double *)(b + p.off[4]);
    st.beta_slot = (float *)(b + p.off[5]); st.rep_of_slot = (int32_t *)(b + p.off[6]); st.slot_of_rep = (int32_t *)(b + p.off[7]);
    st.ladder_id = (int32_t *)(b + p.off[8]); st.n_acc = (int64_t *)(b + p.off[9]); st.n_ex = (int64_t *)(b + p.off[10]);
    std::vector<int32_t> iota(R);
    for (int i = 0; i < R; ++i) iota[i] = i;
    NCE_CUDA(cudaMemcpyAsync(st.sigma, j.sig_src, (size_t)R * j.N, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync((void *)st.beta_slot, j.beta.data(), 4 * (size_t)R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync((void *)st.ladder_id, j.lid.data(), 4 * (size_t)R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.rep_of_slot, iota.data(), 4 * (size_t)R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.slot_of_rep, iota.data(), 4 * (size_t)R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemsetAsync(st.n_acc, 0, 8 * (size_t)R, s));
    NCE_CUDA(cudaMemsetAsync(st.n_ex, 0, 8, s));
    int rc = nce_nce_full_cache((nce_nce_handle)j.d.model, &st, s);
    if (rc) return rc;
    NCE_CUDA(cudaStreamSynchronize(s));
    return NCE_OK;
}

// copy the outputs to the caller's buffers and return the device memory (worker thread, job's stream); the caller
// synchronises the stream, then checks the model's error flags (finish_check)
int finish(SJob &j, cudaStream_t s) {
    const int32_t R = j.d.R;
    const bool ce = j.d.kind == NCE_JOB_CE;
    const int8_t *sig = ce ? j.st.sigma : j.nst.sigma;
    const double *E = ce ? j.st.E : j.nst.E;
    const int64_t *na = ce ? j.st.n_acc : j.nst.n_acc;
    const int32_t *ros = ce ? j.st.rep_of_slot : j.nst.rep_of_slot;
    const int64_t *nx = ce ? j.st.n_ex : j.nst.n_ex;
    if (j.d.sigma_out) NCE_CUDA(cudaMemcpyAsync(j.d.sigma_out, sig, (size_t)R * j.N, cudaMemcpyDeviceToHost, s));
    if (j.d.E_out) NCE_CUDA(cudaMemcpyAsync(j.d.E_out, E, 8 * (size_t)R, cudaMemcpyDeviceToHost, s));
    if (j.d.n_acc_out) NCE_CUDA(cudaMemcpyAsync(j.d.n_acc_out, na, 8 * (size_t)R, cudaMemcpyDeviceToHost, s));
    if (j.d.rep_of_slot_out) NCE_CUDA(cudaMemcpyAsync(j.d.rep_of_slot_out, ros, 4 * (size_t)R, cudaMemcpyDeviceToHost, s));
    if (j.d.n_ex_out) NCE_CUDA(cudaMemcpyAsync(j.d.n_ex_out, nx, 8, cudaMemcpyDeviceToHost, s));
    NCE_CUDA(cudaFreeAsync(j.dev, s));
    return NCE_OK;
}

// a device error flag on the job's model fails the job (the flags stay set for the model's other jobs)
int finish_check(SJob &j) {
    const bool ce = j.d.kind == NCE_JOB_CE;
    int32_t flags = 0;
    const int rc = ce ? ce_error_peek((nce_ce_handle)j.d.model, &flags) : nce_error_peek((nce_nce_handle)j.d.model, &flags);
    if (rc) return rc;
    if (flags) {
        const int code = (flags & 32) ? NCE_ERR_TIMEOUT : NCE_ERR_INVALID;
        return fail(code, "device error flags 0x%x on the job's model: %s", flags, ce ? ce_error_text(flags) : nce_error_text(flags));
    }
    return NCE_OK;
}

void drop(SJob &j, cudaStream_t s) {
    if (j.dev && j.dev != reinterpret_cast<char *>(1)) { cudaFreeAsync(j.dev, s); cudaStreamSynchronize(s); }
}

// io thread of one kind: admit (start) queued jobs that fit and retire finished or cancelled ones
void io_worker(nce_server *S, int kind) {
    cudaSetDevice(S->device);
    cudaStream_t ios = S->io_streams[kind];
    for (;;) {
        std::vector<std::shared_ptr<SJob>> fresh, out;
        std::vector<char> cx;                        // cancelled when taken: a later cancel no longer applies
        {
            std::unique_lock<std::mutex> lk(S->mu);
            for (;;) {
                if (S->stop) return;
                out.assign(S->retiring[kind].begin(), S->retiring[kind].end());
                S->retiring[kind].clear();
                cx.clear();
                for (auto &p : out) cx.push_back(p->cancel ? 1 : 0);
                fresh = admit_locked(S, kind);
                if (!out.empty() || !fresh.empty()) break;
                S->wake.wait_for(lk, std::chrono::milliseconds(2));
            }
        }
        // retire: every finished job's outputs queued on the io stream, one synchronisation, then each job's flags
        std::vector<int> frc(out.size(), NCE_OK);
        for (size_t k = 0; k < out.size(); ++k)
            if (!cx[k]) frc[k] = finish(*out[k], ios);
        if (!out.empty()) {
            const cudaError_t e = cudaStreamSynchronize(ios);
            for (size_t k = 0; k < out.size(); ++k)
                if (!cx[k] && frc[k] == NCE_OK)
                    frc[k] = e != cudaSuccess ? fail(NCE_ERR_CUDA, "retiring a job: %s", cudaGetErrorString(e)) : finish_check(*out[k]);
        }
        for (size_t k = 0; k < out.size(); ++k) {
            SJob &j = *out[k];
            int rc = frc[k];
            if (cx[k]) drop(j, ios);
            std::lock_guard<std::mutex> lk(S->mu);
            j.dev = reinterpret_cast<char *>(1);
            if (cx[k]) {
                release_locked(S, j, NCE_JOB_CANCELLED);
            } else if (rc) {
                j.error = rc; j.msg = last_error();
                release_locked(S, j, NCE_JOB_FAILED);
            } else {
                release_locked(S, j, NCE_JOB_DONE);
            }
        }
        // admit: CE jobs' set-up queued on the io stream for all of them, one synchronisation (host copies of the
        // inputs live in the jobs until then); NeuralCE jobs one at a time on their model's stream
        std::vector<int> src(fresh.size(), NCE_OK);
        if (kind == 0) {
            for (size_t k = 0; k < fresh.size(); ++k) src[k] = start_ce(S, *fresh[k], ios);
            if (!fresh.empty()) {
                const cudaError_t e = cudaStreamSynchronize(ios);
                if (e != cudaSuccess)
                    for (auto &r : src) if (r == NCE_OK) r = fail(NCE_ERR_CUDA, "admitting a job: %s", cudaGetErrorString(e));
            }
        }
        for (size_t k = 0; k < fresh.size(); ++k) {
            auto &p = fresh[k];
            SJob &j = *p;
            int rc;
            cudaStream_t s = ios;
            if (kind == 0) {
                rc = src[k];
            } else {
                // jobs on one model share its scratch buffers, so they share a stream (set-up included)
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    std::shared_ptr<SJob> twin;
                    for (auto &q : S->active[1]) if (q->d.model == j.d.model) twin = q;
                    j.stream = twin ? twin->stream : S->nce_streams[S->rr++ % S->nce_streams.size()];
                }
                s = j.stream;
                rc = start_nce(S, j, s);
            }
            if (rc) {
                drop(j, s);
                j.dev = reinterpret_cast<char *>(1);
                fail_job(S, j, rc);
                continue;
            }
            std::lock_guard<std::mutex> lk(S->mu);
            S->active[kind].push_back(p);
            S->wake.notify_all();
        }
    }
}

// a completed launch: its jobs advance by `steps` (under the lock, where polls read them); finished jobs retire
void end_round(nce_server *S, int kind, std::vector<std::shared_ptr<SJob>> &run, const std::vector<int64_t> &steps) {
    std::lock_guard<std::mutex> lk(S->mu);
    ++S->rounds[kind];
    auto &a = S->active[kind];
    for (size_t i = 0; i < run.size(); ++i) {
        run[i]->done += steps[i];
        S->attempts += steps[i] * run[i]->d.R;
    }
    for (auto &p : run)
        if (p->done >= p->d.n_steps) {
            a.erase(std::remove(a.begin(), a.end(), p), a.end());
            S->retiring[kind].push_back(p);
        }
    S->wake.notify_all();
}

// fail the jobs of a launch that could not be made or did not complete; `s` (the launch's stream) has nothing of
// theirs left in flight.  Their device memory is given back on it (after a device fault that call fails too, and
// the memory stays with the broken context).
void fail_round(nce_server *S, int kind, std::vector<std::shared_ptr<SJob>> &jobs, int rc, cudaStream_t s) {
    std::string m = last_error();
    std::lock_guard<std::mutex> lk(S->mu);
    auto &a = S->active[kind];
    for (auto &p : jobs) {
        if (p->status != NCE_JOB_RUNNING) continue;
        p->error = rc; p->msg = m;
        a.erase(std::remove(a.begin(), a.end(), p), a.end());
        if (p->dev && p->dev != reinterpret_cast<char *>(1)) cudaFreeAsync(p->dev, s);
        release_locked(S, *p, NCE_JOB_FAILED);
    }
}

int64_t chunk_len(const SJob &j) { return std::min(j.d.exchange_every - j.done % j.d.exchange_every, j.d.n_steps - j.done); }

// CE thread: persistent batch launches on a few lanes (one stream each).  Every running CE job that is not in a
// launch joins the next launch on an idle lane (jobs of one cluster order and kernel, at most max_batch a launch),
// and that launch is followed by each job's exact re-anchor; a lane's jobs are free again as soon as its launch
// has completed, so short and long launches do not wait for one another.  A job's chunks (length, Philox key and
// global step) depend only on the job, so its results do not depend on which jobs share its launches.
struct CeLane {
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    std::vector<std::shared_ptr<SJob>> jobs;
    std::vector<int64_t> steps;
    bool busy = false;
};

void ce_worker(nce_server *S) {
    cudaSetDevice(S->device);
    std::vector<CeLane> lanes(S->ce_streams.size());
    for (size_t i = 0; i < lanes.size(); ++i) {
        lanes[i].s = S->ce_streams[i];
        cudaEventCreateWithFlags(&lanes[i].ev, cudaEventDisableTiming);
    }
    std::vector<std::shared_ptr<SJob>> idle;
    for (;;) {
        bool moved = false;
        // 1. completed launches: their jobs advance; finished jobs go to the io thread
        for (auto &ln : lanes) {
            if (!ln.busy) continue;
            const cudaError_t e = cudaEventQuery(ln.ev);
            if (e == cudaErrorNotReady) continue;
            ln.busy = false; moved = true;
            for (auto &p : ln.jobs) p->inflight = false;
            if (e != cudaSuccess) {
                fail_round(S, 0, ln.jobs, fail(NCE_ERR_CUDA, "CE launch: %s", cudaGetErrorString(e)), ln.s);
            } else {
                end_round(S, 0, ln.jobs, ln.steps);
            }
            ln.jobs.clear(); ln.steps.clear();
        }
        // 2. running jobs outside any launch (cancelled ones that are not in a launch leave for the io thread)
        bool any_busy = false;
        for (auto &ln : lanes) any_busy = any_busy || ln.busy;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->stop && !any_busy) break;
            auto &a = S->active[0];
            idle.clear();
            for (auto it = a.begin(); it != a.end();) {
                auto &p = *it;
                if (p->inflight) { ++it; continue; }
                if (p->cancel) { S->retiring[0].push_back(p); it = a.erase(it); S->wake.notify_all(); continue; }
                if (!S->stop) idle.push_back(p);
                ++it;
            }
            if (idle.empty() && !any_busy && !moved) {
                S->wake.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
        }
        // 3. launches of the idle jobs on the idle lanes
        std::map<int32_t, std::vector<std::shared_ptr<SJob>>> by_key;   // one cluster order and kernel a launch
        for (auto &p : idle) by_key[2 * p->mo + p->lf].push_back(p);
        bool launched = false;
        for (auto &grp : by_key) {
            auto &v = grp.second;
            for (size_t a = 0; a < v.size(); a += (size_t)S->cfg.max_batch) {
                CeLane *ln = nullptr;
                for (auto &l : lanes) if (!l.busy) { ln = &l; break; }
                if (!ln) break;
                const int n = (int)std::min<size_t>((size_t)S->cfg.max_batch, v.size() - a);
                std::vector<nce_ce_handle> hs(n); std::vector<nce_pt_state> ss(n); std::vector<nce_pt_chunk> cs(n);
                for (int i = 0; i < n; ++i) {
                    SJob &j = *v[a + i];
                    hs[i] = (nce_ce_handle)j.d.model; ss[i] = j.st;
                    nce_pt_chunk &c = cs[i];
                    std::memset(&c, 0, sizeof(c));
                    c.n_steps = chunk_len(j); c.step0 = j.done; c.seed = j.d.seed; c.sample_interval = 1;
                    c.do_exchange = ((j.done + c.n_steps) % j.d.exchange_every) == 0;
                    c.precision = j.lf ? 64 : S->cfg.precision; c.path = j.lf ? 3 : 0; c.cluster = 1;
                    c.warps = j.lf && S->cfg.ce_lf_warps > 0 ? S->cfg.ce_lf_warps : S->cfg.warps;
                }
                int rc = nce_ce_run_batch(n, hs.data(), ss.data(), cs.data(), ln->s);
                for (int i = 0; i < n && rc == NCE_OK; ++i) {
                    SJob &j = *v[a + i];
                    if (j.st.cv) rc = nce_ce_energy_from_counts(hs[i], j.st.cv, j.d.R, j.st.E, ln->s);
                }
                if (rc == NCE_OK && cudaEventRecord(ln->ev, ln->s) != cudaSuccess) rc = fail(NCE_ERR_CUDA, "CE launch: event record");
                std::vector<std::shared_ptr<SJob>> js(v.begin() + a, v.begin() + a + n);
                if (rc) {
                    // what was enqueued may still run: wait for the lane before the jobs' memory is given back
                    cudaStreamSynchronize(ln->s);
                    fail_round(S, 0, js, rc, ln->s);
                    continue;
                }
                ln->busy = true; launched = true;
                ln->jobs = std::move(js);
                for (int i = 0; i < n; ++i) { ln->jobs[i]->inflight = true; ln->steps.push_back(cs[i].n_steps); }
            }
        }
        if (!launched && !moved) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    for (auto &ln : lanes) {
        if (ln.busy) cudaEventSynchronize(ln.ev);
        cudaEventDestroy(ln.ev);
    }
}

// NeuralCE thread: every running job's next chunk (and its periodic full-cache rebuild) is launched on the job's
// stream as soon as its previous chunk has completed (event query), so jobs of different sizes never wait for one
// another; jobs on one model share a stream, which orders their use of the model's step scratch.
void nce_worker(nce_server *S) {
    cudaSetDevice(S->device);
    std::vector<std::shared_ptr<SJob>> mine, idle;     // jobs with a chunk in flight; jobs ready for the next one
    for (;;) {
        bool moved = false;
        // 1. completed chunks
        for (size_t i = 0; i < mine.size();) {
            auto p = mine[i];
            const cudaError_t e = cudaEventQuery(p->ev);
            if (e == cudaErrorNotReady) { ++i; continue; }
            moved = true;
            p->inflight = false;
            std::vector<std::shared_ptr<SJob>> one{p};
            if (e != cudaSuccess) {
                fail_round(S, 1, one, fail(NCE_ERR_CUDA, "NeuralCE chunk: %s", cudaGetErrorString(e)), p->stream);
            } else {
                end_round(S, 1, one, {p->pending_steps});
            }
            mine[i] = mine.back(); mine.pop_back();
        }
        // 2. running jobs without a chunk in flight (cancelled ones leave for the io thread)
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->stop && mine.empty()) break;
            auto &a = S->active[1];
            idle.clear();
            for (auto it = a.begin(); it != a.end();) {
                auto &p = *it;
                if (p->inflight) { ++it; continue; }
                if (p->cancel) { S->retiring[1].push_back(p); it = a.erase(it); S->wake.notify_all(); continue; }
                if (!S->stop) idle.push_back(p);
                ++it;
            }
            if (idle.empty() && mine.empty() && !moved) {
                S->wake.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
        }
        // 3. the next chunk of each of them
        bool launched = false;
        for (auto &p : idle) {
            SJob &j = *p;
            int rc = NCE_OK;
            if (!j.ev && cudaEventCreateWithFlags(&j.ev, cudaEventDisableTiming) != cudaSuccess)
                rc = fail(NCE_ERR_CUDA, "NeuralCE chunk: event creation");
            nce_nce_chunk c; std::memset(&c, 0, sizeof(c));
            c.n_steps = chunk_len(j); c.step0 = j.done; c.seed = j.d.seed; c.sample_interval = 1;
            c.exchange_rounds = ((j.done + c.n_steps) % j.d.exchange_every) == 0 ? 1 : 0;
            c.cluster = S->cfg.nce_cluster;
            if (!rc) rc = nce_nce_run_chunk((nce_nce_handle)j.d.model, &j.nst, &c, j.stream);
            if (!rc && ++j.chunks % j.anchor == 0) rc = nce_nce_full_cache((nce_nce_handle)j.d.model, &j.nst, j.stream);
            if (!rc && cudaEventRecord(j.ev, j.stream) != cudaSuccess) rc = fail(NCE_ERR_CUDA, "NeuralCE chunk: event record");
            if (rc) {
                cudaStreamSynchronize(j.stream);           // what was enqueued may still run
                std::vector<std::shared_ptr<SJob>> one{p};
                fail_round(S, 1, one, rc, j.stream);
                continue;
            }
            j.pending_steps = c.n_steps; j.inflight = true;
            mine.push_back(p); launched = true;
        }
        if (!launched && !moved) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    for (auto &p : mine) cudaEventSynchronize(p->ev);
}

}  // namespace

extern "C" {

int nce_server_create(const nce_server_config *cfg, nce_server_handle *out) {
    NCE_CHECK(out, "nce_server_create: null argument");
    auto S = std::make_unique<nce_server>();
    if (cfg) S->cfg = *cfg;
    nce_server_config &c = S->cfg;
    if (c.max_batch <= 0) c.max_batch = 64;
    NCE_CHECK(c.max_batch <= 64, "nce_server_create: max_batch must be <= 64");
    if (c.precision == 0) c.precision = 32;
    NCE_CHECK(c.precision == 32 || c.precision == 64, "nce_server_create: precision must be 32 or 64");
    if (c.warps <= 0) c.warps = 8;
    NCE_CHECK(c.warps <= 32, "nce_server_create: warps must be <= 32");
    if (c.nce_cluster <= 0) c.nce_cluster = 1;
    if (c.nce_streams <= 0) c.nce_streams = 4;
    NCE_CHECK(c.nce_streams <= 32, "nce_server_create: nce_streams must be <= 32");
    if (c.starve_s <= 0.0) c.starve_s = 5.0;
    NCE_CUDA(cudaGetDevice(&S->device));
    if (c.hbm_budget <= 0) {
        size_t fr = 0, tot = 0;
        NCE_CUDA(cudaMemGetInfo(&fr, &tot));
        c.hbm_budget = (int64_t)(0.9 * (double)fr);
    }
    for (int k = 0; k < 2; ++k) NCE_CUDA(cudaStreamCreateWithFlags(&S->io_streams[k], cudaStreamNonBlocking));
    for (int i = 0; i < 8; ++i) {                    // CE lanes
        cudaStream_t s;
        NCE_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        S->ce_streams.push_back(s);
    }
    for (int i = 0; i < c.nce_streams; ++i) {
        cudaStream_t s;
        NCE_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        S->nce_streams.push_back(s);
    }
    // keep up to a quarter of the budget of freed job memory in the pool for the next admissions; the rest goes
    // back to the driver, where the models' own allocations can use it
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, S->device) == cudaSuccess) {
        uint64_t keep = (uint64_t)(c.hbm_budget / 4);
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    S->t0 = std::chrono::steady_clock::now();
    nce_server *raw = S.release();
    raw->worker[0] = std::thread(ce_worker, raw);
    raw->worker[1] = std::thread(nce_worker, raw);
    raw->worker[2] = std::thread(io_worker, raw, 0);
    raw->worker[3] = std::thread(io_worker, raw, 1);
    *out = raw;
    return NCE_OK;
}

int nce_server_destroy(nce_server_handle S) {
    if (!S) return NCE_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->wake.notify_all();
    for (auto &w : S->worker) if (w.joinable()) w.join();
    for (int k = 0; k < 2; ++k) {
        for (auto &p : S->active[k]) drop(*p, S->io_streams[k]);
        for (auto &p : S->retiring[k]) drop(*p, S->io_streams[k]);
        cudaStreamDestroy(S->io_streams[k]);
    }
    for (cudaStream_t s : S->ce_streams) cudaStreamDestroy(s);
    for (cudaStream_t s : S->nce_streams) cudaStreamDestroy(s);
    delete S;
    return NCE_OK;
}

int nce_job_submit(nce_server_handle S, const nce_job_desc *d, int64_t *job_id) {
    NCE_CHECK(S && d && job_id, "nce_job_submit: null argument");
    NCE_CHECK(d->kind == NCE_JOB_CE || d->kind == NCE_JOB_NCE, "nce_job_submit: kind must be NCE_JOB_CE or NCE_JOB_NCE");
    NCE_CHECK(d->model && d->R >= 1 && d->sigma && d->beta_slot, "nce_job_submit: model, R, sigma and beta_slot are required");
    NCE_CHECK(d->n_steps >= 1 && d->exchange_every >= 1, "nce_job_submit: n_steps and exchange_every must be >= 1");
    auto j = std::make_shared<SJob>();
    j->d = *d;
    if (d->kind == NCE_JOB_CE) {
        int rc = ce_model_dims((nce_ce_handle)d->model, &j->N, &j->n_cols, &j->mo, &j->binary);
        if (rc) return rc;
        if (S->cfg.ce_kernel == 3 && d->R <= 65535) {
            int32_t ok = 0;
            rc = nce_ce_has_local_field((nce_ce_handle)d->model, &ok, nullptr);
            if (rc) return rc;
            j->lf = ok;
        }
        j->bytes = ce_plan(d->R, j->N, j->n_cols, j->binary != 0, j->lf != 0).total;
        NCE_CHECK(d->R <= 25600, "nce_job_submit: too many replicas for the exchange kernel");
    } else {
        int rc = nce_model_dims((nce_nce_handle)d->model, &j->N, &j->C0, &j->D, &j->depth);
        if (rc) return rc;
        j->bytes = nce_plan(d->R, j->N, j->C0, j->D, j->depth).total;
        j->anchor = d->reanchor_chunks > 0 ? d->reanchor_chunks
                                          : (int32_t)std::max<int64_t>(1, (j->N + d->exchange_every - 1) / d->exchange_every);
    }
    NCE_CHECK((d->flags & ~NCE_JOB_BORROW_SIGMA) == 0, "nce_job_submit: unknown flags 0x%x", d->flags);
    if (d->flags & NCE_JOB_BORROW_SIGMA) {
        j->sig_src = d->sigma;
    } else {
        j->sig.assign(d->sigma, d->sigma + (size_t)d->R * j->N);
        j->sig_src = j->sig.data();
    }
    j->beta.assign(d->beta_slot, d->beta_slot + d->R);
    if (d->ladder_id) j->lid.assign(d->ladder_id, d->ladder_id + d->R);
    else j->lid.assign(d->R, 0);
    j->d.sigma = nullptr; j->d.beta_slot = nullptr; j->d.ladder_id = nullptr;
    std::lock_guard<std::mutex> lk(S->mu);
    if (j->bytes > S->cfg.hbm_budget)
        return fail(NCE_ERR_NOMEM, "nce_job_submit: the job needs %lld bytes of device memory, the budget is %lld",
                    (long long)j->bytes, (long long)S->cfg.hbm_budget);
    j->id = S->next_id++;
    j->t_submit = S->now();
    S->jobs[j->id] = j;
    S->pending[d->kind].push_back(j);
    *job_id = j->id;
    S->wake.notify_all();
    return NCE_OK;
}

int nce_job_poll(nce_server_handle S, int64_t id, nce_job_info *info) {
    NCE_CHECK(S && info, "nce_job_poll: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->jobs.find(id);
    NCE_CHECK(it != S->jobs.end(), "nce_job_poll: unknown job %lld", (long long)id);
    const SJob &j = *it->second;
    info->status = j.status; info->error = j.error; info->steps_done = j.done; info->n_steps = j.d.n_steps;
    info->device_bytes = j.bytes; info->t_submit = j.t_submit; info->t_start = j.t_start; info->t_end = j.t_end;
    return NCE_OK;
}

int nce_job_cancel(nce_server_handle S, int64_t id) {
    NCE_CHECK(S, "nce_job_cancel: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->jobs.find(id);
    NCE_CHECK(it != S->jobs.end(), "nce_job_cancel: unknown job %lld", (long long)id);
    SJob &j = *it->second;
    if (j.status == NCE_JOB_QUEUED || j.status == NCE_JOB_RUNNING) j.cancel = true;
    S->wake.notify_all();
    return NCE_OK;
}

int nce_server_query(nce_server_handle S, nce_server_stats *o) {
    NCE_CHECK(S && o, "nce_server_query: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    o->queued = (int64_t)(S->pending[0].size() + S->pending[1].size());
    o->running = (int64_t)(S->active[0].size() + S->active[1].size() + S->retiring[0].size() + S->retiring[1].size());
    o->done = S->n_done; o->cancelled = S->n_cancelled; o->failed = S->n_failed;
    o->bytes_used = S->bytes_used; o->hbm_budget = S->cfg.hbm_budget;
    o->rounds_ce = S->rounds[0]; o->rounds_nce = S->rounds[1];
    o->attempts = S->attempts.load();
    o->now = S->now();
    return NCE_OK;
}

int nce_job_error(nce_server_handle S, int64_t id, char *buf, size_t n) {
    NCE_CHECK(S && buf && n > 0, "nce_job_error: bad argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->jobs.find(id);
    NCE_CHECK(it != S->jobs.end(), "nce_job_error: unknown job %lld", (long long)id);
    std::snprintf(buf, n, "%s", it->second->msg.c_str());
    return NCE_OK;
}

}  // extern "C"
