// Request server with continuous batching (include/gsgpu.h gsgpu_server_*). No counterpart in the
// reference, which runs one gsPoissonAssembler + gsConjugateGradient per request.
//
// Worker slots each own a context (device buffers, CUDA stream). A free slot takes the head of the
// arrival-ordered queue plus every later queued request with the same dimension and tolerance while
// the batch stays within max_batch requests and the estimated device memory of all running batches
// stays within the budget; it assembles and solves them as one batch (segmented CG). Batches of
// different slots run concurrently on their own streams.
//
// Residency: a slot keeps the contexts of its recent batches (plan, pattern, gather maps and device
// buffers) in a least-recently-used list keyed by the batch's structure (batchSignature). A batch
// whose structure is resident skips refresh(): only its control points and field constants are
// uploaded. Resident contexts count against the budget (admission sees running batches plus
// resident bytes); when the queue head does not fit, the taking slot evicts its own resident
// contexts, and if that is not enough every slot is asked to evict its list.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/gsgpu.h"
#include "context.h"
#include "plan.h"

namespace gsgpu {
namespace {

struct Request {
    long long id = 0;
    ProblemDesc pd;
    std::string sig;  // batchSignature of the request alone
    double tol = 1e-8;
    double est = 0.0;
    bool done = false;
    std::string err;
    std::vector<double> x;
    gsgpu_request_info info{};
};

// device bytes a single-patch request needs in the batch path: the contraction intermediates and
// fields of its layout, the CSR system (upper bound prod_k n_k (2p_k + 1) on its non-zeros) with
// its FP64 values, gather sources, columns, FP32 halves, the half diagonals of the FP32 inner
// operator (at most nnz / 2 + n values), and the solver vectors
double estimateBytes(const ProblemDesc& pd) {
    Layout L;
    buildLayout(pd, L);
    double nnz = 1.0, n = 1.0;
    for (const HostPatch& P : pd.patches)
        for (int k = 0; k < pd.dim; ++k) {
            nnz *= double(P.b[k].n()) * (2 * P.b[k].p + 1);
            n *= double(P.b[k].n());
        }
    const double layout = 8.0 * double(L.s + L.u + L.band + L.fields + L.lfield + L.y1 + L.y2 + L.lv1 + L.lv2 +
                                       L.lvec + L.ntab + L.ngtab + L.npf + 2 * L.coefs);
    return layout + nnz * (8 + 4 + 4 + 2 + 8 + 2) + n * (8 * 12 + 4 * 8 + 4 + 4) + (1 << 20);
}

}  // namespace

struct Resident {
    std::string sig;
    gsgpu_context* ctx = nullptr;
    double bytes = 0.0;
    unsigned long long used = 0;
};

struct Server {
    int device = 0, maxBatch = 64, precision = GSGPU_PREC_MIXED, nslots = 1;
    double budget = 0.0, reserved = 0.0;
    double residentCap = 0.0;   // the most device memory resident contexts may hold (0: none kept)
    double residentBytes = 0.0; // held by resident contexts of all slots
    unsigned long long evictEpoch = 0;  // bumped to ask every slot to evict its resident contexts
    unsigned long long useClock = 0;
    std::mutex m;
    std::condition_variable cvWork, cvDone;
    std::deque<Request*> queue;
    std::map<long long, std::unique_ptr<Request>> reqs;
    std::vector<std::thread> workers;
    bool stop = false;
    long long nextId = 1, nextBatch = 1;
    std::string lastError;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }

    // requests that can never fit fail at once; then the next batch if the head fits (lock held)
    std::vector<Request*> takeBatch() {
        std::vector<Request*> batch;
        while (!queue.empty() && queue.front()->est > budget) {
            Request* r = queue.front();
            queue.pop_front();
            r->info.status = GSGPU_ERR_BUDGET;
            r->err = "request exceeds the device-memory budget of the server";
            r->info.t_start = r->info.t_done = now();
            r->done = true;
            cvDone.notify_all();
        }
        if (queue.empty() || reserved + residentBytes + queue.front()->est > budget) return batch;
        const Request* head = queue.front();
        const int dim = head->pd.dim;
        const double tol = head->tol, quA = head->pd.quA;
        const int quB = head->pd.quB;
        double sum = 0.0;
        for (auto it = queue.begin(); it != queue.end() && int(batch.size()) < maxBatch;) {
            Request* r = *it;
            const bool same = r->pd.dim == dim && r->tol == tol && r->pd.quA == quA && r->pd.quB == quB &&
                              r->pd.dirL2 == head->pd.dirL2;
            if (same && reserved + residentBytes + sum + r->est <= budget) {
                sum += r->est;
                batch.push_back(r);
                it = queue.erase(it);
            } else {
                ++it;
            }
        }
        reserved += sum;
        return batch;
    }

    void work();
    // run the batch on ctx; resident: ctx already holds a refreshed batch of the same structure
    void run(gsgpu_context* ctx, std::vector<Request*>& batch, bool resident);
};

void Server::run(gsgpu_context* ctx, std::vector<Request*>& batch, bool resident) {
    const size_t nb = batch.size();
    std::vector<ProblemDesc> items;
    items.reserve(nb);
    for (Request* r : batch) items.push_back(std::move(r->pd));
    auto clock = [] { return std::chrono::steady_clock::now(); };
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    const auto t0 = clock();
    int rc = GSGPU_OK;
    if (resident) {
        rc = updateBatchData(ctx, items);
    } else {
        rc = setBatchDescs(ctx, items);
        if (rc == GSGPU_OK) rc = gsgpu_refresh(ctx);
    }
    const auto t1 = clock();
    if (rc == GSGPU_OK) rc = gsgpu_assemble(ctx, precision);
    const auto t2 = clock();
    std::vector<double> x;
    std::vector<int> off(nb + 1, 0), its(nb, 0);
    std::vector<double> rr(nb, 0.0);
    if (rc == GSGPU_OK) {
        int nfree = 0, nfixed = 0, nlocal = 0;
        long long nnz = 0;
        rc = gsgpu_sizes(ctx, &nfree, &nnz, &nfixed, &nlocal);
        gsgpu_solver_opts o{};
        o.method = GSGPU_SOLVER_CG_JACOBI;
        o.precision = precision;
        o.tol = batch[0]->tol;
        o.max_iters = 20000;
        o.inner_tol = 1e-5;
        gsgpu_solve_info si{};
        x.assign(size_t(nfree), 0.0);
        if (rc == GSGPU_OK) rc = gsgpu_solve(ctx, &o, x.data(), &si);
        if (rc == GSGPU_ERR_NOT_CONVERGED) rc = GSGPU_OK;  // judged per request below
        if (rc == GSGPU_OK) rc = gsgpu_batch_info(ctx, off.data(), its.data(), rr.data());
    }
    const auto t3 = clock();
    const std::string msg = rc == GSGPU_OK ? std::string() : std::string(gsgpu_last_error(ctx));
    for (size_t j = 0; j < nb; ++j) {
        Request* r = batch[j];
        r->info.batch_size = int(nb);
        r->info.resident = resident ? 1 : 0;
        r->info.ms_setup = ms(t0, t1);
        r->info.ms_assemble = ms(t1, t2);
        r->info.ms_solve = ms(t2, t3);
        if (rc != GSGPU_OK) {
            r->info.status = rc;
            r->err = msg;
            continue;
        }
        r->x.assign(x.begin() + off[j], x.begin() + off[j + 1]);
        r->info.nfree = off[j + 1] - off[j];
        r->info.iterations = its[j];
        r->info.relres = rr[j];
        r->info.status = rr[j] < r->tol ? GSGPU_OK : GSGPU_ERR_NOT_CONVERGED;
        if (r->info.status != GSGPU_OK) r->err = "maximum number of iterations reached";
    }
}

void Server::work() {
#ifdef _OPENMP
    // the slots' host set-up runs concurrently: each gets an equal share of the host threads
    omp_set_num_threads(std::max(1, omp_get_num_procs() / std::max(1, nslots)));
#endif
    std::vector<Resident> mine;  // this slot's resident contexts (least recently used first)
    std::vector<gsgpu_context*> spare;  // contexts without device memory, ready for a new batch
    unsigned long long seenEpoch = 0;
    auto evict = [&](size_t k, std::unique_lock<std::mutex>& lk) {  // lock held on entry and exit
        Resident r = mine[k];
        mine.erase(mine.begin() + long(k));
        residentBytes -= r.bytes;
        lk.unlock();
        releaseDevice(r.ctx);
        spare.push_back(r.ctx);
        lk.lock();
    };
    for (;;) {
        std::vector<Request*> batch;
        gsgpu_context* ctx = nullptr;
        bool resident = false;
        {
            std::unique_lock<std::mutex> lk(m);
            for (;;) {
                if (evictEpoch != seenEpoch) {  // another slot needs the memory of resident contexts
                    seenEpoch = evictEpoch;
                    while (!mine.empty()) evict(0, lk);
                    cvWork.notify_all();
                }
                batch = takeBatch();
                if (!batch.empty() || (stop && queue.empty())) break;
                // the head does not fit: free this slot's resident contexts first, then ask the others
                if (!queue.empty() && reserved + queue.front()->est <= budget &&
                    reserved + residentBytes + queue.front()->est > budget && residentBytes > 0.0) {
                    if (!mine.empty()) {
                        while (!mine.empty()) evict(0, lk);
                        continue;
                    }
                    ++evictEpoch;
                    seenEpoch = evictEpoch;
                    cvWork.notify_all();
                }
                cvWork.wait(lk);
            }
            if (batch.empty()) break;
            const long long bid = nextBatch++;
            const double t = now();
            for (Request* r : batch) {
                r->info.t_start = t;
                r->info.batch_id = bid;
            }
            // a resident context of the same structure takes the batch (its bytes move from the
            // resident count to the batch's reservation)
            std::string sig;
            for (Request* r : batch) sig += r->sig;
            for (size_t k = 0; k < mine.size(); ++k)
                if (mine[k].sig == sig) {
                    ctx = mine[k].ctx;
                    residentBytes -= mine[k].bytes;
                    mine.erase(mine.begin() + long(k));
                    resident = true;
                    break;
                }
            if (!ctx && !spare.empty()) {
                ctx = spare.back();
                spare.pop_back();
            }
            if (!ctx && int(mine.size()) >= 4) {
                // at most four resident contexts per slot before a new handle is made: the least
                // recently used one gives up its memory and its handle takes the batch
                Resident r = mine.front();
                mine.erase(mine.begin());
                residentBytes -= r.bytes;
                lk.unlock();
                releaseDevice(r.ctx);
                lk.lock();
                ctx = r.ctx;
            }
        }
        int crc = GSGPU_OK;
        if (!ctx) crc = gsgpu_create(&ctx, device);
        if (crc != GSGPU_OK) {
            for (Request* r : batch) {
                r->info.status = crc;
                r->err = "could not create a CUDA context for the server slot";
            }
            ctx = nullptr;
        } else {
            std::string sig;
            for (Request* r : batch) sig += r->sig;
            run(ctx, batch, resident);
            // keep the context resident when its memory fits the resident cap, else release it
            const double bytes = deviceBytes(ctx);
            std::unique_lock<std::mutex> lk(m);
            bool keep = residentCap > 0.0 && bytes <= residentCap && batch[0]->info.status == GSGPU_OK;
            while (keep && residentBytes + bytes > residentCap && !mine.empty()) evict(0, lk);
            keep = keep && residentBytes + bytes <= residentCap;
            if (keep) {
                mine.push_back(Resident{sig, ctx, bytes, ++useClock});
                residentBytes += bytes;
                ctx = nullptr;
            }
        }
        if (ctx) {
            releaseDevice(ctx);  // not kept: an idle slot holds no device memory for it
            spare.push_back(ctx);
        }
        {
            std::lock_guard<std::mutex> lk(m);
            double sum = 0.0;
            const double t = now();
            for (Request* r : batch) {
                sum += r->est;
                r->info.t_done = t;
                r->done = true;
            }
            reserved -= sum;
        }
        cvDone.notify_all();
        cvWork.notify_all();
    }
    {
        std::unique_lock<std::mutex> lk(m);
        while (!mine.empty()) evict(0, lk);
    }
    for (gsgpu_context* c : spare) gsgpu_destroy(c);
}

}  // namespace gsgpu

struct gsgpu_server {
    gsgpu::Server s;
};

extern "C" {

int gsgpu_server_create(gsgpu_server** out, int device, int slots, double budget_bytes, int max_batch, int precision) {
    if (!out || slots < 1 || budget_bytes <= 0 || max_batch < 1 ||
        (precision != GSGPU_PREC_FP64 && precision != GSGPU_PREC_MIXED))
        return GSGPU_ERR_INVALID;
    gsgpu_server* p = new gsgpu_server();
    p->s.device = device;
    p->s.budget = budget_bytes;
    p->s.maxBatch = max_batch;
    p->s.precision = precision;
    p->s.nslots = slots;
    p->s.residentCap = 0.25 * budget_bytes;  // default: a quarter of the budget for resident batches
    for (int i = 0; i < slots; ++i) p->s.workers.emplace_back([p] { p->s.work(); });
    *out = p;
    return GSGPU_OK;
}

int gsgpu_server_submit(gsgpu_server* srv, const gsgpu_problem* prob, double tol, long long* id) {
    if (!srv || !prob || !id) return GSGPU_ERR_INVALID;
    gsgpu::Server& S = srv->s;
    std::unique_ptr<gsgpu::Request> r(new gsgpu::Request());
    try {
        gsgpu::problemFromC(prob, r->pd);
        if (r->pd.patches.size() != 1 || !r->pd.ifaces.empty())
            throw std::invalid_argument("server requests must be single patches without interfaces");
        r->est = gsgpu::estimateBytes(r->pd);
        r->sig = gsgpu::batchSignature(std::vector<gsgpu::ProblemDesc>(1, r->pd));
    } catch (const std::exception& e) {
        std::lock_guard<std::mutex> lk(S.m);
        S.lastError = e.what();
        return GSGPU_ERR_INVALID;
    }
    r->tol = tol > 0 ? tol : 1e-8;
    r->info.est_bytes = r->est;
    {
        std::lock_guard<std::mutex> lk(S.m);
        if (S.stop) return GSGPU_ERR_STATE;
        r->info.t_submit = S.now();
        r->id = S.nextId++;
        *id = r->id;
        S.queue.push_back(r.get());
        S.reqs[r->id] = std::move(r);
    }
    S.cvWork.notify_one();
    return GSGPU_OK;
}

int gsgpu_server_wait(gsgpu_server* srv, long long id, double* x, int capacity, gsgpu_request_info* info) {
    if (!srv) return GSGPU_ERR_INVALID;
    gsgpu::Server& S = srv->s;
    std::unique_lock<std::mutex> lk(S.m);
    auto it = S.reqs.find(id);
    if (it == S.reqs.end()) {
        S.lastError = "unknown request id";
        return GSGPU_ERR_INVALID;
    }
    gsgpu::Request* r = it->second.get();
    S.cvDone.wait(lk, [&] { return r->done; });
    if (x && capacity < int(r->x.size())) {
        S.lastError = "solution buffer too small";
        return GSGPU_ERR_INVALID;
    }
    if (info) *info = r->info;
    if (x) std::copy(r->x.begin(), r->x.end(), x);
    const int status = r->info.status;
    if (status != GSGPU_OK) S.lastError = r->err;
    S.reqs.erase(it);
    return status;
}

int gsgpu_server_set_resident(gsgpu_server* srv, double bytes) {
    if (!srv || bytes < 0.0) return GSGPU_ERR_INVALID;
    std::lock_guard<std::mutex> lk(srv->s.m);
    if (bytes > srv->s.budget) return GSGPU_ERR_INVALID;
    srv->s.residentCap = bytes;
    if (srv->s.residentBytes > bytes) ++srv->s.evictEpoch;  // slots give up their lists
    srv->s.cvWork.notify_all();
    return GSGPU_OK;
}

const char* gsgpu_server_last_error(const gsgpu_server* srv) { return srv ? srv->s.lastError.c_str() : "null server"; }

int gsgpu_server_destroy(gsgpu_server* srv) {
    if (!srv) return GSGPU_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(srv->s.m);
        srv->s.stop = true;
    }
    srv->s.cvWork.notify_all();
    for (std::thread& t : srv->s.workers) t.join();
    delete srv;
    return GSGPU_OK;
}

}  // extern "C"
