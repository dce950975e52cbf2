// Request server: continuous batching of independent Newton-step solves on
// one GPU (the C ABI's idp_server_*). Host-only C++: a FIFO of jobs, an
// admission rule on the sum of the admitted jobs' memory footprints, and a
// pool of worker threads; each worker owns one context (one CUDA stream and
// one device arena) and solves one cohort at a time, so cohorts of different
// workers overlap on the device. New jobs are admitted whenever a worker is
// free and the budget allows, i.e. while other cohorts are between Newton
// iterations. The reference has no counterpart: its Python driver advances
// one scene per call (Python/Drivers/FEMDiscreteShellBase.py:333-361).
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

#include "idp_gb300.h"

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
    idp_job_info info{};
};

using Clock = std::chrono::steady_clock;

}  // namespace

struct idp_server {
    idp_params P{};
    double budget = 0;
    int max_batch = 1;
    bool simulated = false;
    double sim_ms_per_kvertex = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job*> pending;
    std::map<int, std::unique_ptr<Job>> jobs;
    int next_id = 0;
    int next_cohort = 0;
    double resident = 0;          // sum of footprints of admitted, unfinished jobs
    std::vector<double> held;     // device bytes each worker's context holds
    bool stop = false;
    int running = 0;
    idp_server_stats st{};
    std::vector<std::thread> threads;
    Clock::time_point t0 = Clock::now();

    double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
    bool admissible() const { return !pending.empty() && resident + pending.front()->footprint <= budget; }
};

namespace {

// One cohort on a worker's context: add, commit, predictors, advance, read back.
int solve_cohort(idp_server* S, idp_ctx*& ctx, std::vector<Job*>& cohort, std::vector<idp_result>& res) {
    int rc = IDP_OK;
    if (!ctx) {
        ctx = idp_create(&S->P, &rc);
        if (!ctx) return rc ? rc : IDP_ERR_CUDA;
    } else if ((rc = idp_reset(ctx))) {
        return rc;
    }
    for (Job* j : cohort) {
        int k = idp_add_instance(ctx, j->V, j->X.data(), j->X0.data(), j->T, j->tets.data(), j->mass.data(),
                                 j->lam.data(), j->mu.data(), j->nDBC, j->dbc.empty() ? nullptr : j->dbc.data(),
                                 j->dHat2, j->kappa, j->kappa_max);
        if (k < 0) return -k;
        if (j->has_v && (rc = idp_set_velocity(ctx, k, j->v.data()))) return rc;
    }
    if ((rc = idp_commit(ctx))) return rc;
    for (size_t k = 0; k < cohort.size(); ++k)
        if (cohort[k]->normal_flow != 0 && (rc = idp_set_normal_flow(ctx, (int)k, cohort[k]->normal_flow))) return rc;
    res.assign(cohort.size(), idp_result{});
    rc = idp_advance(ctx, res.data());
    if (rc == IDP_ERR_CUDA || rc == IDP_ERR_CAPACITY || rc == IDP_ERR_STATE || rc == IDP_ERR_INVALID_ARG) return rc;
    for (size_t k = 0; k < cohort.size(); ++k) {
        Job* j = cohort[k];
        if (j->X_out || j->v_out) {
            int r = idp_get_state(ctx, (int)k, j->X_out, j->v_out, nullptr);
            if (r) return r;
        }
    }
    return IDP_OK;
}

void simulate_cohort(idp_server* S, std::vector<Job*>& cohort, std::vector<idp_result>& res) {
    double kv = 0;
    for (Job* j : cohort) kv += j->V / 1000.0;
    std::this_thread::sleep_for(std::chrono::duration<double, std::milli>(S->sim_ms_per_kvertex * kv));
    res.assign(cohort.size(), idp_result{});
    for (size_t k = 0; k < cohort.size(); ++k) {
        Job* j = cohort[k];
        res[k].status = IDP_OK;
        res[k].newton_iters = 1;
        if (j->X_out) std::copy(j->X.begin(), j->X.end(), j->X_out);
        if (j->v_out) std::fill(j->v_out, j->v_out + 3 * (size_t)j->V, 0.0);
    }
}

void worker(idp_server* S, int w) {
    idp_ctx* ctx = nullptr;
    std::unique_lock<std::mutex> lk(S->mu);
    while (true) {
        S->cv_work.wait(lk, [&] { return S->admissible() || (S->stop && S->pending.empty()); });
        if (S->pending.empty()) break;  // stopping, nothing left
        // cohort: jobs from the head of the queue while they fit
        std::vector<Job*> cohort;
        double fp = 0;
        while (!S->pending.empty() && (int)cohort.size() < S->max_batch &&
               S->resident + fp + S->pending.front()->footprint <= S->budget) {
            fp += S->pending.front()->footprint;
            cohort.push_back(S->pending.front());
            S->pending.pop_front();
        }
        S->resident += fp;
        S->st.peak_resident = std::max(S->st.peak_resident, S->resident);
        S->running += 1;
        S->st.peak_concurrency = std::max(S->st.peak_concurrency, S->running);
        const int cid = S->next_cohort++;
        S->st.cohorts += 1;
        const double t_admit = S->now_ms();
        for (Job* j : cohort) {
            j->info.admit_ms = t_admit;
            j->info.cohort = cid;
            j->info.cohort_size = (int)cohort.size();
        }
        if (!S->pending.empty()) S->cv_work.notify_one();  // another worker may take the rest
        lk.unlock();

        std::vector<idp_result> res;
        int rc = IDP_OK;
        try {
            if (S->simulated) simulate_cohort(S, cohort, res);
            else rc = solve_cohort(S, ctx, cohort, res);
        } catch (const std::bad_alloc&) {
            rc = IDP_ERR_CAPACITY;  // host memory for the cohort's arrays
        } catch (...) {
            rc = IDP_ERR_INVALID_ARG;
        }
        if (rc == IDP_OK && res.size() != cohort.size()) rc = IDP_ERR_STATE;
        size_t bytes = 0;
        if (ctx) idp_device_bytes(ctx, &bytes);

        lk.lock();
        const double t_done = S->now_ms();
        for (size_t k = 0; k < cohort.size(); ++k) {
            Job* j = cohort[k];
            j->info.result = rc == IDP_OK ? res[k] : idp_result{};
            j->info.status = rc == IDP_OK ? res[k].status : rc;
            j->info.result.status = j->info.status;
            j->info.done_ms = t_done;
            j->done = true;
            // the record stays for idp_server_wait; the inputs are no longer needed
            std::vector<double>().swap(j->X);
            std::vector<double>().swap(j->X0);
            std::vector<double>().swap(j->mass);
            std::vector<double>().swap(j->lam);
            std::vector<double>().swap(j->mu);
            std::vector<double>().swap(j->v);
            std::vector<int32_t>().swap(j->tets);
            std::vector<int32_t>().swap(j->dbc);
        }
        S->resident -= fp;
        S->running -= 1;
        S->st.completed += (long long)cohort.size();
        // keep the context's buffers for the next cohort while all workers'
        // contexts together stay under the budget
        S->held[w] = (double)bytes;
        double total = 0;
        for (double h : S->held) total += h;
        if (ctx && (total > S->budget || rc == IDP_ERR_CUDA)) {
            lk.unlock();
            idp_destroy(ctx);
            ctx = nullptr;
            lk.lock();
            S->held[w] = 0;
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
    lk.unlock();
    if (ctx) idp_destroy(ctx);
}

idp_server* make_server(double budget, int workers, int max_batch) {
    if (!(budget > 0) || workers < 1 || max_batch < 1) return nullptr;
    idp_server* S = new idp_server();
    idp_default_params(&S->P);
    S->budget = budget;
    S->max_batch = max_batch;
    S->held.assign(workers, 0.0);
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
