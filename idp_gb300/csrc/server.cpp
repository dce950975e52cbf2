// Request server: continuous batching of independent Newton-step solves on
// one GPU (the C ABI's idp_server_*). Host C++: a FIFO of jobs, an admission
// rule on device memory, and a pool of worker threads; each worker owns one
// context (one CUDA stream and one device arena) holding the jobs it is
// solving. A worker advances its jobs a few Newton iterations at a time
// (step_iterate); between those chunks it releases every job that finished
// (its result is written at once) and, once half of its slots are free,
// admits jobs from the head of the queue into its running arena: the jobs
// still iterating are snapshotted, the arena is rebuilt with them and the new
// jobs, and their Newton loops resume where they were. Workers run concurrently on their own streams. The
// reference has no counterpart: its Python driver advances one scene per
// call (Python/Drivers/FEMDiscreteShellBase.py:333-361).
//
// Memory: a worker occupies max(bytes its context holds, footprints of its
// unfinished jobs); a job is admitted only while the sum of that over all
// workers, with the job added to the admitting worker, stays within the
// budget. An idle worker's context counts too: when the head job does not fit
// and some idle worker holds memory, the idle workers are asked to give
// their contexts back.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "engine.hpp"

namespace {

struct Job {
    int id = 0;
    int V = 0, T = 0, nDBC = 0;
    std::vector<double> X, X0, mass, lam, mu, v;
    std::vector<int32_t> tets, dbc;
    double dHat2 = 0, kappa = 0, kappa_max = 0, normal_flow = 0;
    bool has_v = false;
    double* X_out = nullptr;
    double* v_out = nullptr;
    double footprint = 0;
    bool done = false;
    std::shared_ptr<idp::HostInstance> host;  // built at its first admission, reused by later re-packs
    int sim_left = 0;  // simulated mode: Newton iterations still to run
    idp_job_info info{};
};

using Clock = std::chrono::steady_clock;

// simulated mode: a job of V vertices needs 2 + V/1000 Newton iterations; an
// iteration of a worker costs ms_per_kvertex / 10 per thousand vertices of
// its unfinished jobs
int sim_iters(int V) { return 2 + V / 1000; }

}  // namespace

struct idp_server {
    idp_params P{};
    double budget = 0;
    int max_batch = 1;
    int chunk = 8;                // Newton iterations between admission points
    bool simulated = false;
    double sim_ms_per_kvertex = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job*> pending;
    std::map<int, std::unique_ptr<Job>> jobs;
    int next_id = 0;
    int next_cohort = 0;
    std::vector<double> held;     // device bytes each worker's context holds
    std::vector<double> res;      // footprints of each worker's unfinished jobs
    std::vector<int> live;        // each worker's unfinished jobs
    bool release_req = false;     // the head job waits for idle workers' memory
    bool stop = false;
    idp_server_stats st{};
    std::vector<std::thread> threads;
    Clock::time_point t0 = Clock::now();

    double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
    double occupied(int w, double extra) const { return std::max(held[w], res[w] + extra); }
    // device memory in use if worker w took `extra` more bytes of jobs
    double total_with(int w, double extra) const {
        double t = 0;
        for (size_t k = 0; k < held.size(); ++k) t += occupied((int)k, (int)k == w ? extra : 0.0);
        return t;
    }
    bool head_fits(int w) const {
        return !pending.empty() && live[w] < max_batch && total_with(w, pending.front()->footprint) <= budget;
    }
    void note_peaks() {
        double r = 0;
        int running = 0;
        for (size_t k = 0; k < res.size(); ++k) {
            r += res[k];
            running += live[k] > 0;
        }
        st.peak_resident = std::max(st.peak_resident, r);
        st.peak_device = std::max(st.peak_device, total_with(-1, 0.0));
        st.peak_concurrency = std::max(st.peak_concurrency, running);
    }
};

namespace {

// A worker's arena and the jobs in it, in arena order; slots of finished jobs
// stay (inactive) until the next re-pack.
struct Slots {
    idp_ctx* ctx = nullptr;
    std::vector<Job*> job;
    std::vector<char> live;
    std::vector<idp_result> res;
    double sim_bytes = 0;  // simulated mode: bytes the arena would hold
};

// Rebuild the worker's arena with its unfinished jobs (resumed where their
// Newton loops were) followed by the new jobs (begun).
int repack(idp_server* S, Slots& W, const std::vector<Job*>& fresh) {
    std::vector<Job*> keep;
    std::vector<idp::InstSnapshot> snaps;
    int rc;
    for (size_t k = 0; k < W.job.size(); ++k)
        if (W.live[k]) {
            keep.push_back(W.job[k]);
            if (!S->simulated) {
                snaps.emplace_back();
                if ((rc = idp::snapshot_instance(W.ctx, (int)k, snaps.back()))) return rc;
            }
        }
    W.job = keep;
    W.job.insert(W.job.end(), fresh.begin(), fresh.end());
    W.live.assign(W.job.size(), 1);
    W.res.assign(W.job.size(), idp_result{});
    if (S->simulated) {
        double fp = 0;
        for (Job* j : W.job) fp += j->footprint;
        W.sim_bytes = std::max(W.sim_bytes, fp);  // grow-only, as a real context
        return IDP_OK;
    }
    if (!W.ctx) {
        W.ctx = idp_create(&S->P, &rc);
        if (!W.ctx) return rc ? rc : IDP_ERR_CUDA;
    } else if ((rc = idp_reset(W.ctx))) {
        return rc;
    }
    for (Job* j : W.job) {
        // a carried-over job's instance is re-added from its cached copy
        // (no second surface extraction; its state comes from the snapshot)
        int k = j->host ? idp::add_prebuilt(W.ctx, *j->host)
                        : idp_add_instance(W.ctx, j->V, j->X.data(), j->X0.data(), j->T, j->tets.data(),
                                           j->mass.data(), j->lam.data(), j->mu.data(), j->nDBC,
                                           j->dbc.empty() ? nullptr : j->dbc.data(), j->dHat2, j->kappa, j->kappa_max);
        if (k < 0) return -k;
        if (k >= (int)keep.size() && j->has_v && (rc = idp_set_velocity(W.ctx, k, j->v.data()))) return rc;
    }
    if ((rc = idp_commit(W.ctx))) return rc;
    for (size_t k = keep.size(); k < W.job.size(); ++k)
        if (!W.job[k]->host) W.job[k]->host = std::make_shared<idp::HostInstance>(*idp::instance_host(W.ctx, (int)k));
    for (size_t k = 0; k < keep.size(); ++k)
        if ((rc = idp::resume_instance(W.ctx, (int)k, snaps[k]))) return rc;
    std::vector<unsigned char> which(W.job.size(), 0);
    for (size_t k = keep.size(); k < W.job.size(); ++k) {
        which[k] = 1;
        Job* j = W.job[k];
        if (j->normal_flow != 0 && (rc = idp_set_normal_flow(W.ctx, (int)k, j->normal_flow))) return rc;
    }
    if ((rc = idp::step_begin(W.ctx, which))) return rc;
    return idp::step_prepare_resumed(W.ctx);
}

// One chunk of Newton iterations of the worker's live jobs.
int iterate(idp_server* S, Slots& W) {
    if (S->simulated) {
        double kv = 0;
        for (size_t k = 0; k < W.job.size(); ++k)
            if (W.live[k]) kv += W.job[k]->V / 1000.0;
        int n = 0;
        for (size_t k = 0; k < W.job.size(); ++k)
            if (W.live[k]) n = std::max(n, std::min(S->chunk, W.job[k]->sim_left));
        std::this_thread::sleep_for(std::chrono::duration<double, std::milli>(S->sim_ms_per_kvertex * kv * n / 10.0));
        for (size_t k = 0; k < W.job.size(); ++k) {
            if (!W.live[k]) continue;
            Job* j = W.job[k];
            j->sim_left -= std::min(n, j->sim_left);
            W.res[k].newton_iters = sim_iters(j->V) - j->sim_left;
            W.res[k].status = j->sim_left > 0 ? IDP_ERR_NOT_CONVERGED : IDP_OK;
        }
        return IDP_OK;
    }
    int left = 0;
    const int rc = idp::step_iterate(W.ctx, S->chunk, W.res.data(), &left);
    if (rc == IDP_ERR_CUDA || rc == IDP_ERR_CAPACITY || rc == IDP_ERR_STATE || rc == IDP_ERR_INVALID_ARG) return rc;
    return IDP_OK;
}

// true when slot k's job stopped iterating
bool finished(idp_server* S, Slots& W, size_t k) {
    if (S->simulated) return W.job[k]->sim_left <= 0;
    return !idp::instance_active(W.ctx, (int)k);
}

void release_inputs(Job* j) {
    std::vector<double>().swap(j->X);
    std::vector<double>().swap(j->X0);
    std::vector<double>().swap(j->mass);
    std::vector<double>().swap(j->lam);
    std::vector<double>().swap(j->mu);
    std::vector<double>().swap(j->v);
    std::vector<int32_t>().swap(j->tets);
    std::vector<int32_t>().swap(j->dbc);
}

double held_bytes(idp_server* S, Slots& W) {
    if (S->simulated) return W.sim_bytes;
    size_t bytes = 0;
    if (W.ctx) idp_device_bytes(W.ctx, &bytes);
    return (double)bytes;
}

void drop_context(Slots& W) {
    if (W.ctx) idp_destroy(W.ctx);
    W.ctx = nullptr;
    W.sim_bytes = 0;
    W.job.clear();
    W.live.clear();
    W.res.clear();
}

void worker(idp_server* S, int w) {
    Slots W;
    std::unique_lock<std::mutex> lk(S->mu);
    while (true) {
        S->cv_work.wait(lk, [&] {
            return S->live[w] > 0 || S->head_fits(w) || (S->release_req && S->live[w] == 0 && S->held[w] > 0) ||
                   (S->stop && S->pending.empty());
        });
        if (S->live[w] == 0 && S->pending.empty() && S->stop) break;
        if (S->live[w] == 0 && !S->head_fits(w)) {
            // idle, asked to give its memory back
            lk.unlock();
            drop_context(W);
            lk.lock();
            S->held[w] = 0;
            S->cv_work.notify_all();
            continue;
        }
        // admission at the queue head, between Newton iterations; a worker
        // that is iterating admits once half of its slots are free (each
        // admission rebuilds its arena, so admissions are batched)
        std::vector<Job*> fresh;
        double fp = 0;
        const bool may_admit = S->live[w] == 0 || S->max_batch - S->live[w] >= std::max(1, S->max_batch / 2);
        while (may_admit && !S->pending.empty() && S->live[w] + (int)fresh.size() < S->max_batch &&
               S->total_with(w, fp + S->pending.front()->footprint) <= S->budget) {
            fp += S->pending.front()->footprint;
            fresh.push_back(S->pending.front());
            S->pending.pop_front();
        }
        if (!fresh.empty()) {
            S->res[w] += fp;
            S->live[w] += (int)fresh.size();
            S->release_req = false;
            const int cid = S->next_cohort++;
            S->st.cohorts += 1;
            const double t_admit = S->now_ms();
            for (Job* j : fresh) {
                j->info.admit_ms = t_admit;
                j->info.cohort = cid;
                j->sim_left = sim_iters(j->V);
            }
            S->note_peaks();
        }
        // the head job waits for memory that idle workers hold: ask them
        if (!S->pending.empty() && fresh.empty() && !S->head_fits(w)) {
            for (size_t k = 0; k < S->held.size(); ++k)
                if ((int)k != w && S->live[k] == 0 && S->held[k] > 0) S->release_req = true;
            if (S->release_req) S->cv_work.notify_all();
        }
        if (!S->pending.empty()) S->cv_work.notify_one();  // another worker may take the rest
        lk.unlock();

        int rc = IDP_OK;
        try {
            if (!fresh.empty()) rc = repack(S, W, fresh);
            for (Job* j : fresh) j->info.cohort_size = (int)W.job.size();
            if (rc == IDP_OK) rc = iterate(S, W);
        } catch (const std::bad_alloc&) {
            rc = IDP_ERR_CAPACITY;  // host memory for the jobs' arrays
        } catch (...) {
            rc = IDP_ERR_INVALID_ARG;
        }
        // results of the jobs that stopped (all live jobs on an error)
        std::vector<size_t> done;
        for (size_t k = 0; k < W.job.size(); ++k)
            if (W.live[k] && (rc != IDP_OK || finished(S, W, k))) done.push_back(k);
        std::vector<int> out_rc(done.size(), IDP_OK);
        for (size_t d = 0; d < done.size(); ++d) {
            Job* j = W.job[done[d]];
            if (rc == IDP_OK && !S->simulated && (j->X_out || j->v_out))
                out_rc[d] = idp_get_state(W.ctx, (int)done[d], j->X_out, j->v_out, nullptr);
            if (rc == IDP_OK && S->simulated) {
                if (j->X_out) std::copy(j->X.begin(), j->X.end(), j->X_out);
                if (j->v_out) std::fill(j->v_out, j->v_out + 3 * (size_t)j->V, 0.0);
            }
        }
        const double bytes = held_bytes(S, W);

        lk.lock();
        const double t_done = S->now_ms();
        for (size_t d = 0; d < done.size(); ++d) {
            const size_t k = done[d];
            Job* j = W.job[k];
            const int status = rc != IDP_OK ? rc : (out_rc[d] != IDP_OK ? out_rc[d] : W.res[k].status);
            j->info.result = rc == IDP_OK ? W.res[k] : idp_result{};
            j->info.status = status;
            j->info.result.status = status;
            j->info.result.latency_ms = t_done - j->info.admit_ms;
            j->info.done_ms = t_done;
            j->done = true;
            W.live[k] = 0;
            S->res[w] -= j->footprint;
            S->live[w] -= 1;
            S->st.completed += 1;
            release_inputs(j);
        }
        if (S->live[w] == 0) S->res[w] = 0;  // no rounding residue
        S->held[w] = bytes;
        S->note_peaks();
        if (rc == IDP_ERR_CUDA || (S->live[w] == 0 && S->total_with(-1, 0.0) > S->budget)) {
            lk.unlock();
            drop_context(W);
            lk.lock();
            S->held[w] = 0;
        }
        if (!done.empty()) S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
    lk.unlock();
    drop_context(W);
}

idp_server* make_server(double budget, int workers, int max_batch) {
    if (!(budget > 0) || workers < 1 || max_batch < 1) return nullptr;
    idp_server* S = new idp_server();
    idp_default_params(&S->P);
    S->budget = budget;
    S->max_batch = max_batch;
    S->held.assign(workers, 0.0);
    S->res.assign(workers, 0.0);
    S->live.assign(workers, 0);
    return S;
}

void start(idp_server* S, int workers) {
    for (int w = 0; w < workers; ++w) S->threads.emplace_back(worker, S, w);
}

}  // namespace

extern "C" {

double idp_job_footprint(int V, int T) {
    // per vertex: positions and solver vectors (FP64 and FP32), BSR rows of
    // the tet stencil (about 15 blocks of FP32 and FP64 values), contact and
    // CCD lists; per tet: element data, contributor lists, element Hessians;
    // plus the fixed broad-phase tables
    return 4096.0 * V + 1792.0 * T + 48.0e6;
}

idp_server* idp_server_create(const idp_params* p, double hbm_budget, int workers, int max_batch, int* status) {
    idp_server* S = make_server(hbm_budget, workers, max_batch);
    if (!S) {
        if (status) *status = IDP_ERR_INVALID_ARG;
        return nullptr;
    }
    if (p) S->P = *p;
    start(S, workers);
    if (status) *status = IDP_OK;
    return S;
}

idp_server* idp_server_create_simulated(double hbm_budget, int workers, int max_batch, double ms_per_kvertex,
                                        int* status) {
    idp_server* S = make_server(hbm_budget, workers, max_batch);
    if (!S || !(ms_per_kvertex >= 0)) {
        delete S;
        if (status) *status = IDP_ERR_INVALID_ARG;
        return nullptr;
    }
    S->simulated = true;
    S->sim_ms_per_kvertex = ms_per_kvertex;
    start(S, workers);
    if (status) *status = IDP_OK;
    return S;
}

int idp_server_submit(idp_server* S, const idp_job_desc* d) {
    if (!S || !d || d->V <= 0 || d->T <= 0 || !d->X || !d->tets || !d->mass || !d->lam || !d->mu)
        return -IDP_ERR_INVALID_ARG;
    auto j = std::make_unique<Job>();
    j->V = d->V;
    j->T = d->T;
    j->X.assign(d->X, d->X + 3 * (size_t)d->V);
    j->X0.assign(d->X0 ? d->X0 : d->X, (d->X0 ? d->X0 : d->X) + 3 * (size_t)d->V);
    j->tets.assign(d->tets, d->tets + 4 * (size_t)d->T);
    j->mass.assign(d->mass, d->mass + d->V);
    j->lam.assign(d->lam, d->lam + d->T);
    j->mu.assign(d->mu, d->mu + d->T);
    j->nDBC = d->nDBC > 0 && d->dbc_idx ? d->nDBC : 0;
    if (j->nDBC) j->dbc.assign(d->dbc_idx, d->dbc_idx + j->nDBC);
    j->dHat2 = d->dHat2;
    j->kappa = d->kappa;
    j->kappa_max = d->kappa_max;
    j->has_v = d->v != nullptr;
    if (j->has_v) j->v.assign(d->v, d->v + 3 * (size_t)d->V);
    j->normal_flow = d->normal_flow;
    j->X_out = d->X_out;
    j->v_out = d->v_out;
    j->footprint = idp_job_footprint(d->V, d->T);
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return -IDP_ERR_STATE;
    if (j->footprint > S->budget) return -IDP_ERR_CAPACITY;
    j->id = S->next_id++;
    j->info.submit_ms = S->now_ms();
    j->info.footprint = j->footprint;
    Job* raw = j.get();
    S->jobs[j->id] = std::move(j);
    S->pending.push_back(raw);
    S->st.submitted += 1;
    S->cv_work.notify_one();
    return raw->id;
}

int idp_server_wait(idp_server* S, int id, idp_job_info* info) {
    if (!S) return IDP_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->jobs.find(id);
    if (it == S->jobs.end()) return IDP_ERR_INVALID_ARG;
    Job* j = it->second.get();
    S->cv_done.wait(lk, [&] { return j->done; });
    if (info) *info = j->info;
    return IDP_OK;
}

int idp_server_drain(idp_server* S) {
    if (!S) return IDP_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv_done.wait(lk, [&] { return S->st.completed == S->st.submitted; });
    return IDP_OK;
}

int idp_server_get_stats(idp_server* S, idp_server_stats* out) {
    if (!S || !out) return IDP_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    *out = S->st;
    double h = 0;
    for (double b : S->held) h += b;
    out->device_bytes = h;
    return IDP_OK;
}

void idp_server_destroy(idp_server* S) {
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (auto& t : S->threads) t.join();
    delete S;
}

}  // extern "C"
