// Serving: whole DMRG runs as requests, with continuous batching of their
// ground-state solves.
//
// A request is one finite-DMRG run (init_dmrg + finite_DMRG,
// src/DMRG_MAIN.f90:140-241) of its own model, length and bond dimension.
// The server
//   * admits queued requests while the sum of their estimated HBM footprints
//     stays within its budget (one request always runs, whatever its
//     estimate), first come first served;
//   * runs every admitted request on a worker thread with its own context,
//     so block enlargement, superblock set-up and the host side of the
//     renormalisation of different requests overlap, while their block
//     state (operator pool, Krylov basis, rho blocks) stays resident in HBM
//     for the request's life;
//   * sends every mixed-precision ground-state solve of every request to one
//     batch engine (the persistent multi-solve Lanczos kernel): a
//     dispatcher thread adds solves as they arrive and runs one round of all
//     solves in flight at a time, so the H*psi products of different
//     requests share each launch;
//   * serialises the device phases of the workers (superblock upload, RDM,
//     device renormalisation) and the dispatcher's rounds with one lock, so
//     the cooperative kernels of one never wait on the other's.
// FP64 requests solve on their own context (under the lock); they get the
// admission and the overlap of host work, not the batching.  No counterpart
// in the reference (its runs are one per MPI job).
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <system_error>
#include <thread>
#include <vector>

#include "device.cuh"
#include "host_dmrg.hpp"

namespace nss {

struct Server;

namespace {

using clk = std::chrono::steady_clock;

struct Job {                      // one ground-state solve waiting for the dispatcher
    Ctx *c = nullptr;
    uint64_t seed = 0;
    int nitermax = 0;
    double tol = 0.0;
    bool done = false, direct = false;
    int rc = 0, numop = 0;
    double energy = 0.0;
};

struct Request {
    int id = 0;
    nss_dmrg_params p{};
    std::vector<int32_t> msweep;
    std::vector<double> esweep;
    size_t footprint = 0;
    clk::time_point t_submit, t_admit, t_done;
    int status = 0;
    double energy = 0.0;          // final ground-state energy per site
    size_t peak_bytes = 0;        // the context's largest device allocation total
};

}  // namespace

struct Server {
    int device = 0;
    size_t budget = 0, in_use = 0, peak_in_use = 0;
    nss_ctx *host = nullptr;      // owns the batch engine's stream and barrier
    BatchEngine *eng = nullptr;
    std::mutex mu;                // queues, counters, results
    std::condition_variable cv;   // admission and dispatcher wake-ups
    std::condition_variable cv_job;
    std::mutex gpu;               // device phases and engine rounds, one at a time
    std::deque<std::shared_ptr<Request>> pending;
    std::vector<std::shared_ptr<Request>> finished;
    std::deque<Job *> submitted;
    std::map<int, Job *> inflight;
    int running = 0, next_id = 1;
    bool stop = false;
    std::vector<std::thread> workers;
    std::thread admitter, dispatcher;
    std::atomic<int64_t> rounds{0}, batched_solves{0}, solves{0};
    double solves_in_flight_sum = 0.0;
};

namespace {

void run_request(Server *S, std::shared_ptr<Request> r) {
    nss_ctx *ctx = nss_create(S->device, 0);
    int rc = ctx ? NSS_OK : NSS_ERR_CUDA;
    if (ctx) {
        Ctx &c = ctx_of(ctx);
        c.serve = S;
        nss_dmrg_params p = r->p;
        p.msweep = r->msweep.empty() ? nullptr : r->msweep.data();
        p.esweep = r->esweep.empty() ? nullptr : r->esweep.data();
        nss_dmrg *d = nss_dmrg_create(ctx, &p);
        if (!d) rc = NSS_ERR_INVALID;
        else {
            rc = nss_dmrg_finite(d);
            const int nrec = nss_dmrg_nrecords(d);
            if (!rc && nrec > 0) {
                std::vector<nss_step_record> recs(nrec);
                nss_dmrg_records(d, recs.data(), nrec);
                r->energy = recs.back().energy[0];
            }
            nss_dmrg_destroy(d);
        }
        r->peak_bytes = c.peak_used;
        nss_destroy(ctx);
    }
    std::lock_guard<std::mutex> lk(S->mu);
    r->status = rc;
    r->t_done = clk::now();
    S->in_use -= r->footprint;
    --S->running;
    S->finished.push_back(r);
    S->cv.notify_all();
}

void admit_loop(Server *S) {
    std::unique_lock<std::mutex> lk(S->mu);
    while (true) {
        S->cv.wait(lk, [&] {
            if (S->stop && S->pending.empty()) return true;
            if (S->pending.empty()) return false;
            return S->running == 0 || S->in_use + S->pending.front()->footprint <= S->budget;
        });
        if (S->pending.empty()) break;
        auto r = S->pending.front();
        S->pending.pop_front();
        r->t_admit = clk::now();
        try {
            S->workers.emplace_back(run_request, S, r);
        } catch (const std::system_error &) {   // no thread for it: the request fails, the server goes on
            r->status = NSS_ERR_NOMEM;
            r->t_done = clk::now();
            S->finished.push_back(r);
            continue;
        }
        S->in_use += r->footprint;
        S->peak_in_use = std::max(S->peak_in_use, S->in_use);
        ++S->running;
    }
}

void dispatch_loop(Server *S) {
    std::vector<int> ids(256), nops(256);
    std::vector<double> es(256);
    std::unique_lock<std::mutex> lk(S->mu);
    while (true) {
        S->cv.wait(lk, [&] {
            return !S->submitted.empty() || !S->inflight.empty() || (S->stop && S->running == 0);
        });
        if (S->submitted.empty() && S->inflight.empty()) break;   // stopped, every request done
        std::deque<Job *> jobs;
        jobs.swap(S->submitted);
        lk.unlock();
        std::vector<Job *> released;
        int nd = 0;
        {
            std::lock_guard<std::mutex> g(S->gpu);
            for (Job *j : jobs) {
                int id = 0;
                const int rc = batch_add(S->eng, *j->c, j->seed, j->nitermax, j->tol, &id);
                if (rc) {                 // the worker solves it on its own context
                    j->direct = true;
                    released.push_back(j);
                } else {
                    std::lock_guard<std::mutex> l2(S->mu);
                    S->inflight[id] = j;
                }
            }
            const int nin = batch_inflight(S->eng);
            if (nin > 0) {
                S->solves_in_flight_sum += nin;
                ++S->rounds;
                const int rc = batch_step(S->eng, 256, &nd, ids.data(), es.data(), nops.data());
                if (rc) {                 // a failed round: its solves go back to their workers
                    std::lock_guard<std::mutex> l2(S->mu);
                    for (auto &kv : S->inflight) {
                        kv.second->direct = true;
                        released.push_back(kv.second);
                    }
                    S->inflight.clear();
                    nd = 0;
                }
            }
        }
        lk.lock();
        for (int q = 0; q < nd; ++q) {
            auto it = S->inflight.find(std::abs(ids[q]));
            if (it == S->inflight.end()) continue;
            Job *j = it->second;
            S->inflight.erase(it);
            if (ids[q] > 0) {
                j->energy = es[q];
                j->numop = nops[q];
                ++S->batched_solves;
            } else {
                j->direct = true;
            }
            released.push_back(j);
        }
        for (Job *j : released) j->done = true;
        if (!released.empty()) S->cv_job.notify_all();
    }
}

}  // namespace

// The device lock of a served context (no-op otherwise).
ServeLock::ServeLock(Ctx &c) : s(c.serve) {
    if (s) s->gpu.lock();
}
ServeLock::~ServeLock() { unlock(); }
void ServeLock::unlock() {
    if (s) s->gpu.unlock();
    s = nullptr;
}

void serve_count(Ctx &c) {
    if (c.serve) ++c.serve->solves;
}

int serve_solve(Ctx &c, int nitermax, double tol, uint64_t seed, double *energy, int *numop) {
    Server *S = c.serve;
    Job j;
    j.c = &c;
    j.seed = seed;
    j.nitermax = nitermax;
    j.tol = tol;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        S->submitted.push_back(&j);
        S->cv.notify_all();
        S->cv_job.wait(lk, [&] { return j.done; });
    }
    if (j.direct) {                   // not batched: on the worker's own context
        ServeLock g(c);
        return lanczos_eigh(c, 1, nitermax, tol, seed, NSS_PREC_MIXED, energy, numop);
    }
    *energy = j.energy;
    *numop = j.numop;
    c.last_numop = j.numop;
    return NSS_OK;
}

size_t serve_footprint(const nss_dmrg_params &p, const int32_t *msweep, int nsweep) {
    const int d = p.model == NSS_MODEL_HUBBARD ? 4 : (p.model == NSS_MODEL_HEISENBERG_ONE ? 3 : 2);
    int m = p.mdmrg;
    for (int i = 0; i < nsweep; ++i) m = std::max(m, (int)msweep[i]);
    const double M = (double)m * d * 1.1;          // enlarged block (+ degeneracy extensions)
    // the largest superblock: the first finite step enlarges an unrenormalised
    // block once more (src/DMRG_MAIN.f90:302-306), N ~ 0.6 d M^2 at most
    const double n = 0.6 * d * M * M;
    const int nit = p.lanc_niter > 0 ? p.lanc_niter : 512;
    const double basis = (p.precision == NSS_PREC_MIXED ? 4.0 : 8.0) * (nit + 1) * n;
    const double vectors = 200.0 * n;              // work vectors, Ritz vectors, refinement scratch
    const double ops = 90.0 * M * M * d;           // sector operators (FP64 + FP32 + tensor-core planes), rho blocks
    const double fixed = 64.0 * (1 << 20);         // per-context buffers sized by the GPU (partial sums, tables)
    return (size_t)(basis + vectors + ops + fixed);
}

}  // namespace nss

using nss::Server;

extern "C" {

nss_server *nss_server_create(int device, size_t hbm_budget) {
    auto *S = new (std::nothrow) Server;
    if (!S) return nullptr;
    S->device = device;
    S->budget = hbm_budget;
    S->host = nss_create(device, 0);
    if (!S->host) {
        delete S;
        return nullptr;
    }
    try {
        S->eng = nss::batch_create(nss::ctx_of(S->host));
    } catch (const std::exception &) {
        S->eng = nullptr;
    }
    if (!S->eng) {
        nss_destroy(S->host);
        delete S;
        return nullptr;
    }
    try {
        S->admitter = std::thread(nss::admit_loop, S);
        S->dispatcher = std::thread(nss::dispatch_loop, S);
    } catch (const std::system_error &) {   // no threads: no server (nothing was submitted yet)
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->stop = true;
            S->cv.notify_all();
        }
        if (S->admitter.joinable()) S->admitter.join();
        nss::batch_destroy(S->eng);
        nss_destroy(S->host);
        delete S;
        return nullptr;
    }
    return (nss_server *)S;
}

size_t nss_server_footprint(const nss_dmrg_params *p) {
    return p ? nss::serve_footprint(*p, p->msweep, p->nsweep) : 0;
}

int nss_server_submit(nss_server *sv, const nss_dmrg_params *p, int *id) {
    auto *S = (Server *)sv;
    if (!S || !p || !id) return NSS_ERR_INVALID;
    if (p->lanc_neigen > 1) return NSS_ERR_INVALID;   // the engine solves ground states
    try {
        auto r = std::make_shared<nss::Request>();
        r->p = *p;
        if (p->msweep && p->nsweep > 0) r->msweep.assign(p->msweep, p->msweep + p->nsweep);
        if (p->esweep && p->nsweep > 0) r->esweep.assign(p->esweep, p->esweep + p->nsweep);
        r->p.lanc_neigen = 1;
        r->footprint = nss::serve_footprint(*p, p->msweep, p->nsweep);
        r->t_submit = nss::clk::now();
        std::lock_guard<std::mutex> lk(S->mu);
        r->id = S->next_id++;
        *id = r->id;
        S->pending.push_back(r);
        S->cv.notify_all();
    } catch (const std::bad_alloc &) {
        return NSS_ERR_NOMEM;
    }
    return NSS_OK;
}

int nss_server_poll(nss_server *sv, int max, nss_served *out) {
    auto *S = (Server *)sv;
    if (!S || (max > 0 && !out)) return NSS_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    int n = 0;
    while (n < max && !S->finished.empty()) {
        auto r = S->finished.front();
        S->finished.erase(S->finished.begin());
        nss_served &o = out[n++];
        o.id = r->id;
        o.status = r->status;
        o.energy = r->energy;
        o.wait_s = std::chrono::duration<double>(r->t_admit - r->t_submit).count();
        o.service_s = std::chrono::duration<double>(r->t_done - r->t_admit).count();
        o.footprint_est = r->footprint;
        o.peak_bytes = r->peak_bytes;
    }
    return n;
}

int nss_server_stats(nss_server *sv, int *queued, int *running, size_t *in_use, size_t *peak_in_use,
                     int64_t *rounds, double *mean_batch) {
    auto *S = (Server *)sv;
    if (!S) return NSS_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    if (queued) *queued = (int)S->pending.size();
    if (running) *running = S->running;
    if (in_use) *in_use = S->in_use;
    if (peak_in_use) *peak_in_use = S->peak_in_use;
    if (rounds) *rounds = S->rounds;
    if (mean_batch) *mean_batch = S->rounds ? S->solves_in_flight_sum / (double)S->rounds : 0.0;
    return NSS_OK;
}

int64_t nss_server_solves(nss_server *sv) { return sv ? ((Server *)sv)->solves.load() : 0; }

void nss_server_destroy(nss_server *sv) {
    auto *S = (Server *)sv;
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        S->cv.notify_all();
    }
    S->admitter.join();          // every queued request admitted
    for (auto &t : S->workers) t.join();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->cv.notify_all();
    }
    S->dispatcher.join();
    nss::batch_destroy(S->eng);
    nss_destroy(S->host);
    delete S;
}

}  // extern "C"
