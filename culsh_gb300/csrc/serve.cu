// Serving loop: continuous batching of kNN requests over one device-resident
// index (no counterpart in the reference, whose SearchTables::search is one
// synchronous call per query set, cuLSH_SearchTables.cu:197-463).
//
// Host code only, layered on the public search API. A server owns a pool of
// slots; each slot is one search object with its own CUDA stream, device and
// pinned host buffers, and worker thread, so that batches in different slots
// run on the device at the same time. A scheduler thread forms batches as
// slots free up: the oldest pending request plus later ones with the same
// (K, T), up to max_batch_queries queries, and admits a batch when the device
// bytes of all slots (their search buffers, which grow to the largest search
// they ran, plus the slot's query/result buffers) stay within the memory
// budget; idle slots give their buffers back when that makes room. A batch
// larger than the budget is cut back to its first request; a request that
// alone exceeds the budget fails with CULSH_ERR_OUT_OF_MEMORY, as the
// reference's admission check fails a query whose candidates do not fit
// (cuLSH_SearchTables.cu:303-306). Results are exact: a request's ids and
// distances do not depend on the batch it ran in.
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

#include "culsh.h"
#include "culsh_internal.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    unsigned long long ticket = 0;
    const float* queries = nullptr;
    int Q = 0, K = 0, T = 0;
    int* out_ids = nullptr;
    float* out_d = nullptr;
    Clock::time_point t_submit;
    bool done = false;
    int status = CULSH_OK;
    std::string err;
};
using ReqPtr = std::shared_ptr<Request>;

struct Slot {
    culsh_search* s = nullptr;
    cudaStream_t st = nullptr;
    int K = 0, T = 0;                      // the search object's current reset
    float* d_q = nullptr;
    int* d_ids = nullptr;
    float* d_d = nullptr;
    float* h_q = nullptr;                  // pinned staging
    int* h_ids = nullptr;
    float* h_d = nullptr;
    size_t cap_q = 0;                      // query rows the buffers hold
    size_t cap_o = 0, cap_k = 0;           // result buffers hold cap_o * cap_k entries
    std::vector<ReqPtr> batch;
    bool busy = false;
    long long reserved = 0;                // device bytes held by this slot
    std::condition_variable cv;
    std::thread worker;
};

}  // namespace

struct culsh_server {
    culsh_index* ix = nullptr;
    int D = 0, L = 0;
    int n_slots = 4, max_batch = 8192, graphs = 0;
    long long budget = 0;
    std::mutex mu;
    std::condition_variable cv_sched, cv_done;
    std::deque<ReqPtr> pending;
    std::map<unsigned long long, ReqPtr> live;   // submitted, not yet collected
    std::vector<std::unique_ptr<Slot>> slots;
    std::thread scheduler;
    bool stop = false;
    unsigned long long next_ticket = 1;
    int in_flight = 0;
    // statistics
    std::vector<double> lat_ms;
    long long n_req = 0, n_q = 0, n_batches = 0, n_failed = 0, peak_bytes = 0;
    int max_in_flight = 0;
    bool have_first = false;
    Clock::time_point t_first, t_last;
};

namespace {

long long slot_buffer_bytes(size_t q_rows, size_t o_rows, size_t k, int D) {
    return (long long)(q_rows * (size_t)D * 4 + o_rows * k * 8);
}

long long total_reserved(culsh_server* v) {
    long long b = 0;
    for (auto& sl : v->slots) b += sl->reserved;
    return b;
}

// Grows the slot's query and result buffers for a batch of Q queries with K
// neighbours (device and pinned host). Runs under the library's allocation
// lock so that no other slot is capturing a graph meanwhile.
int ensure_slot_buffers(Slot* sl, size_t Q, size_t K, int D) {
    std::lock_guard<std::mutex> lk(culsh::alloc_capture_mutex());
    if (Q > sl->cap_q) {
        cudaFree(sl->d_q);
        cudaFreeHost(sl->h_q);
        sl->d_q = nullptr;
        sl->h_q = nullptr;
        sl->cap_q = 0;
        if (cudaMalloc(&sl->d_q, Q * D * sizeof(float)) != cudaSuccess ||
            cudaMallocHost(&sl->h_q, Q * D * sizeof(float)) != cudaSuccess)
            return culsh::set_last_error(CULSH_ERR_OUT_OF_MEMORY, "serving: query buffers could not be allocated");
        sl->cap_q = Q;
    }
    if (Q * K > sl->cap_o * sl->cap_k) {   // results are Q x K, row-major
        cudaFree(sl->d_ids);
        cudaFree(sl->d_d);
        cudaFreeHost(sl->h_ids);
        cudaFreeHost(sl->h_d);
        sl->d_ids = nullptr;
        sl->d_d = nullptr;
        sl->h_ids = nullptr;
        sl->h_d = nullptr;
        sl->cap_o = sl->cap_k = 0;
        const size_t n = Q * K;
        if (cudaMalloc(&sl->d_ids, n * 4) != cudaSuccess || cudaMalloc(&sl->d_d, n * 4) != cudaSuccess ||
            cudaMallocHost(&sl->h_ids, n * 4) != cudaSuccess || cudaMallocHost(&sl->h_d, n * 4) != cudaSuccess)
            return culsh::set_last_error(CULSH_ERR_OUT_OF_MEMORY, "serving: result buffers could not be allocated");
        sl->cap_o = Q;
        sl->cap_k = K;
    }
    return CULSH_OK;
}

void free_slot(Slot* sl) {
    std::lock_guard<std::mutex> lk(culsh::alloc_capture_mutex());
    cudaFree(sl->d_q);
    cudaFree(sl->d_ids);
    cudaFree(sl->d_d);
    cudaFreeHost(sl->h_q);
    cudaFreeHost(sl->h_ids);
    cudaFreeHost(sl->h_d);
    sl->d_q = nullptr;
    sl->d_ids = nullptr;
    sl->d_d = nullptr;
    sl->h_q = nullptr;
    sl->h_ids = nullptr;
    sl->h_d = nullptr;
    sl->cap_q = sl->cap_o = sl->cap_k = 0;
}

// One batch on one slot: stage the queries, search, scatter the results.
int run_batch(culsh_server* v, Slot* sl, const std::vector<ReqPtr>& batch) {
    const int K = batch[0]->K, T = batch[0]->T, D = v->D;
    size_t Q = 0;
    for (auto& r : batch) Q += (size_t)r->Q;
    int rc = ensure_slot_buffers(sl, Q, (size_t)K, D);
    if (rc != CULSH_OK) return rc;
    size_t row = 0;
    for (auto& r : batch) {
        std::memcpy(sl->h_q + row * D, r->queries, (size_t)r->Q * D * sizeof(float));
        row += (size_t)r->Q;
    }
    if (cudaMemcpyAsync(sl->d_q, sl->h_q, Q * D * sizeof(float), cudaMemcpyHostToDevice, sl->st) != cudaSuccess)
        return culsh::set_last_error(CULSH_ERR_CUDA, "serving: query upload failed");
    if (sl->K != K || sl->T != T) {
        rc = culsh_search_reset(sl->s, v->ix, K, T);
        if (rc != CULSH_OK) return rc;
        sl->K = K;
        sl->T = T;
    }
    rc = culsh_search_run_device(sl->s, sl->d_q, (int)Q, sl->d_ids, sl->d_d, sl->st);
    if (rc != CULSH_OK) return rc;
    if (cudaMemcpyAsync(sl->h_ids, sl->d_ids, Q * K * 4, cudaMemcpyDeviceToHost, sl->st) != cudaSuccess ||
        cudaMemcpyAsync(sl->h_d, sl->d_d, Q * K * 4, cudaMemcpyDeviceToHost, sl->st) != cudaSuccess ||
        cudaStreamSynchronize(sl->st) != cudaSuccess)
        return culsh::set_last_error(CULSH_ERR_CUDA, "serving: result download failed");
    row = 0;
    for (auto& r : batch) {
        std::memcpy(r->out_ids, sl->h_ids + row * K, (size_t)r->Q * K * 4);
        std::memcpy(r->out_d, sl->h_d + row * K, (size_t)r->Q * K * 4);
        row += (size_t)r->Q;
    }
    return CULSH_OK;
}

void worker_loop(culsh_server* v, Slot* sl) {
    for (;;) {
        std::vector<ReqPtr> batch;
        {
            std::unique_lock<std::mutex> lk(v->mu);
            sl->cv.wait(lk, [&] { return sl->busy || v->stop; });
            if (!sl->busy) return;   // stopping and idle
            batch = sl->batch;
        }
        const int rc = run_batch(v, sl, batch);
        const std::string err = rc == CULSH_OK ? std::string() : std::string(culsh_last_error());
        const long long held = culsh_search_device_bytes(sl->s) + slot_buffer_bytes(sl->cap_q, sl->cap_o, sl->cap_k, v->D);
        const Clock::time_point now = Clock::now();
        {
            std::lock_guard<std::mutex> lk(v->mu);
            for (auto& r : batch) {
                r->done = true;
                r->status = rc;
                r->err = err;
                ++v->n_req;
                if (rc == CULSH_OK) {
                    v->n_q += r->Q;
                    v->lat_ms.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
                } else {
                    ++v->n_failed;
                }
            }
            ++v->n_batches;
            v->t_last = now;
            sl->batch.clear();
            sl->busy = false;
            sl->reserved = held;
            --v->in_flight;
            v->peak_bytes = std::max(v->peak_bytes, total_reserved(v));
        }
        v->cv_done.notify_all();
        v->cv_sched.notify_all();
    }
}

void fail_request(culsh_server* v, const ReqPtr& r, int code, const std::string& msg) {
    r->done = true;
    r->status = code;
    r->err = msg;
    ++v->n_req;
    ++v->n_failed;
}

void scheduler_loop(culsh_server* v) {
    std::unique_lock<std::mutex> lk(v->mu);
    for (;;) {
        auto idle = [&]() -> Slot* {
            for (auto& sl : v->slots)
                if (!sl->busy) return sl.get();
            return nullptr;
        };
        v->cv_sched.wait(lk, [&] { return v->stop || (!v->pending.empty() && idle()); });
        if (v->pending.empty()) {
            if (v->stop) return;
            continue;
        }
        // Batch: the oldest request plus later ones with the same (K, T).
        const ReqPtr r0 = v->pending.front();
        std::vector<ReqPtr> batch{r0};
        size_t Qb = (size_t)r0->Q;
        for (size_t i = 1; i < v->pending.size(); ++i) {
            const ReqPtr& r = v->pending[i];
            if (r->K == r0->K && r->T == r0->T && Qb + (size_t)r->Q <= (size_t)v->max_batch) {
                batch.push_back(r);
                Qb += (size_t)r->Q;
            }
        }
        // Slot: an idle one already reset to (K, T) keeps its graph and buffers.
        Slot* sl = nullptr;
        for (auto& s : v->slots)
            if (!s->busy && s->K == r0->K && s->T == r0->T) {
                sl = s.get();
                break;
            }
        if (!sl) sl = idle();
        auto need_of = [&](size_t q) {
            return culsh_search_estimate_bytes(v->ix, (int)q, r0->K, r0->T) +
                   slot_buffer_bytes(q, q, (size_t)r0->K, v->D);
        };
        long long need = need_of(Qb);
        auto fits = [&]() { return total_reserved(v) - sl->reserved + std::max(need, sl->reserved) <= v->budget; };
        if (!fits()) {
            // Idle slots give their buffers back, largest first.
            std::vector<Slot*> idle_slots;
            for (auto& s : v->slots)
                if (!s->busy && s.get() != sl && s->reserved > 0) idle_slots.push_back(s.get());
            std::sort(idle_slots.begin(), idle_slots.end(), [](Slot* a, Slot* b) { return a->reserved > b->reserved; });
            for (Slot* s : idle_slots) {
                if (fits()) break;
                culsh_search_release(s->s);
                free_slot(s);
                s->reserved = 0;
                s->K = s->T = 0;
            }
        }
        if (!fits() && sl->reserved > need_of(Qb)) {
            // The chosen slot holds more than this batch needs: start it afresh.
            culsh_search_release(sl->s);
            free_slot(sl);
            sl->reserved = 0;
            sl->K = sl->T = 0;
        }
        if (!fits() && batch.size() > 1) {
            batch.resize(1);
            Qb = (size_t)r0->Q;
            need = need_of(Qb);
        }
        if (!fits()) {
            if (need > v->budget) {   // never fits, even alone on an idle device
                v->pending.pop_front();
                char msg[256];
                snprintf(msg, sizeof msg,
                         "serving: request %llu needs %lld device bytes, more than the budget %lld",
                         r0->ticket, need, v->budget);
                fail_request(v, r0, CULSH_ERR_OUT_OF_MEMORY, msg);
                v->cv_done.notify_all();
                continue;
            }
            // Wait for a running batch to finish and give memory back.
            v->cv_sched.wait(lk, [&] { return v->stop || v->in_flight == 0 || fits(); });
            continue;
        }
        for (const ReqPtr& r : batch) {
            auto it = std::find(v->pending.begin(), v->pending.end(), r);
            if (it != v->pending.end()) v->pending.erase(it);
        }
        sl->batch = batch;
        sl->busy = true;
        sl->reserved = std::max(sl->reserved, need);
        ++v->in_flight;
        v->max_in_flight = std::max(v->max_in_flight, v->in_flight);
        v->peak_bytes = std::max(v->peak_bytes, total_reserved(v));
        sl->cv.notify_one();
    }
}

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * (double)(v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int culsh_server_create(culsh_server** out, culsh_index* ix, const culsh_server_config* cfg) {
    if (!out || !ix) return culsh::set_last_error(CULSH_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    int rc = culsh::index_make_resident(ix);
    if (rc != CULSH_OK) return rc;
    auto v = std::make_unique<culsh_server>();
    v->ix = ix;
    int N = 0, M = 0;
    float W = 0.0f;
    culsh_index_params(ix, &N, &v->D, &v->L, &M, &W);
    if (cfg) {
        if (cfg->slots < 0 || cfg->slots > 64 || cfg->max_batch_queries < 0 || cfg->memory_budget < 0)
            return culsh::set_last_error(CULSH_ERR_INVALID_ARGUMENT, "serving: configuration out of range");
        if (cfg->slots) v->n_slots = cfg->slots;
        if (cfg->max_batch_queries) v->max_batch = cfg->max_batch_queries;
        v->budget = cfg->memory_budget;
        v->graphs = cfg->graphs != 0;
    }
    if (v->budget == 0) {
        size_t freeb = 0, totalb = 0;
        if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess)
            return culsh::set_last_error(CULSH_ERR_CUDA, "serving: cudaMemGetInfo failed");
        v->budget = (long long)(0.8 * (double)freeb);
    }
    for (int i = 0; i < v->n_slots; ++i) {
        auto sl = std::make_unique<Slot>();
        if (culsh_search_create(&sl->s) != CULSH_OK ||
            cudaStreamCreateWithFlags(&sl->st, cudaStreamNonBlocking) != cudaSuccess) {
            for (auto& s : v->slots) {
                culsh_search_destroy(s->s);
                cudaStreamDestroy(s->st);
            }
            if (sl->s) culsh_search_destroy(sl->s);
            return culsh::set_last_error(CULSH_ERR_CUDA, "serving: slot creation failed");
        }
        culsh_search_set_graphs(sl->s, v->graphs);
        culsh_search_set_profiling(sl->s, 0);   // latency is measured per request on the host
        v->slots.push_back(std::move(sl));
    }
    culsh_server* p = v.release();
    for (auto& sl : p->slots) sl->worker = std::thread(worker_loop, p, sl.get());
    p->scheduler = std::thread(scheduler_loop, p);
    *out = p;
    return CULSH_OK;
}

int culsh_server_submit(culsh_server* v, const float* queries, int Q, int K, int T, int* out_ids, float* out_dists,
                        unsigned long long* ticket) {
    if (!v || !queries || !out_ids || !out_dists || !ticket)
        return culsh::set_last_error(CULSH_ERR_INVALID_ARGUMENT, "null argument");
    if (Q <= 0 || K <= 0 || T <= 0)
        return culsh::set_last_error(CULSH_ERR_INVALID_ARGUMENT, "Integer parameters must be all positive.");
    if (K > CULSH_MAX_K || T > CULSH_MAX_T)
        return culsh::set_last_error(CULSH_ERR_CAPACITY, "serving: K or T beyond the supported maximum");
    auto r = std::make_shared<Request>();
    r->queries = queries;
    r->Q = Q;
    r->K = K;
    r->T = T;
    r->out_ids = out_ids;
    r->out_d = out_dists;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(v->mu);
        if (v->stop) return culsh::set_last_error(CULSH_ERR_STATE, "serving: the server is shutting down");
        r->ticket = v->next_ticket++;
        if (!v->have_first) {
            v->have_first = true;
            v->t_first = r->t_submit;
        }
        v->pending.push_back(r);
        v->live[r->ticket] = r;
        *ticket = r->ticket;
    }
    v->cv_sched.notify_all();
    return CULSH_OK;
}

int culsh_server_wait(culsh_server* v, unsigned long long ticket, double timeout_s) {
    if (!v) return culsh::set_last_error(CULSH_ERR_INVALID_ARGUMENT, "null server");
    std::unique_lock<std::mutex> lk(v->mu);
    auto it = v->live.find(ticket);
    if (it == v->live.end()) return culsh::set_last_error(CULSH_ERR_INVALID_ARGUMENT, "serving: unknown ticket");
    ReqPtr r = it->second;
    auto pred = [&] { return r->done; };
    if (timeout_s < 0) {
        v->cv_done.wait(lk, pred);
    } else if (!v->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
        return CULSH_PENDING;
    }
    v->live.erase(ticket);
    if (r->status != CULSH_OK) return culsh::set_last_error(r->status, r->err.c_str());
    return CULSH_OK;
}

int culsh_server_stats_get(culsh_server* v, culsh_server_stats* out) {
    if (!v || !out) return culsh::set_last_error(CULSH_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(v->mu);
    *out = culsh_server_stats{};
    out->requests = v->n_req;
    out->queries = v->n_q;
    out->batches = v->n_batches;
    out->failed = v->n_failed;
    out->wall_s = v->have_first ? std::chrono::duration<double>(v->t_last - v->t_first).count() : 0.0;
    out->qps = out->wall_s > 0 ? (double)v->n_q / out->wall_s : 0.0;
    out->p50_ms = percentile(v->lat_ms, 0.50);
    out->p99_ms = percentile(v->lat_ms, 0.99);
    double sum = 0.0, mx = 0.0;
    for (double x : v->lat_ms) {
        sum += x;
        mx = std::max(mx, x);
    }
    out->mean_ms = v->lat_ms.empty() ? 0.0 : sum / (double)v->lat_ms.size();
    out->max_ms = mx;
    out->max_in_flight = v->max_in_flight;
    out->peak_device_bytes = v->peak_bytes;
    out->budget_bytes = v->budget;
    out->slots = v->n_slots;
    return CULSH_OK;
}

int culsh_server_stats_reset(culsh_server* v) {
    if (!v) return culsh::set_last_error(CULSH_ERR_INVALID_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lk(v->mu);
    v->lat_ms.clear();
    v->n_req = v->n_q = v->n_batches = v->n_failed = 0;
    v->max_in_flight = v->in_flight;
    v->peak_bytes = total_reserved(v);
    v->have_first = false;
    return CULSH_OK;
}

void culsh_server_destroy(culsh_server* v) {
    if (!v) return;
    {   // drain: every submitted request completes first
        std::unique_lock<std::mutex> lk(v->mu);
        v->cv_done.wait(lk, [&] { return v->pending.empty() && v->in_flight == 0; });
        v->stop = true;
    }
    v->cv_sched.notify_all();
    for (auto& sl : v->slots) sl->cv.notify_all();
    if (v->scheduler.joinable()) v->scheduler.join();
    for (auto& sl : v->slots)
        if (sl->worker.joinable()) sl->worker.join();
    for (auto& sl : v->slots) {
        culsh_search_destroy(sl->s);
        free_slot(sl.get());
        cudaStreamDestroy(sl->st);
    }
    delete v;
}

}  // extern "C"
