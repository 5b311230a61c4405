// Serving loop: continuous batching of search requests over one resident index.
//
// Requests (1..n queries, their own k and ef) are queued by gsx_server_submit.  A dispatcher
// thread admits queued requests, oldest first, into a fixed arena of device query slots (each
// slot holds one query row, its results and status); a group of requests takes one contiguous
// range of slots, and admission stops when the arena has no free range for the next request, so
// device memory bounds the work in flight.  Every admitted group is launched at once on a free
// stream: one copy in per array over the group's range, one persistent search launch over the
// group (its queries addressed through a slot list), one copy out per array, and a host callback
// that marks the group done, so the dispatcher's work per group does not grow with the number
// of requests in it.  Groups on different streams overlap on the device, and requests that arrive while
// others run are admitted as soon as slots and a stream free up.  The search arithmetic is the
// batched kernel's, so a query's result does not depend on what it ran with.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <cmath>
#include <random>
#include <vector>

#include "gsx_host.h"
#include "gsx_ranges.h"

namespace gsx {
int server_make_cfg(gsx_searcher *s, int kmax, int efmax, int nq, LaunchCfg *cfg, int *spill_bits);
int server_resolve_one(gsx_searcher *s, const float *q, int k, int ef, int32_t *ids, float *dis);
}  // namespace gsx

using namespace gsx;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    int nq = 0, k = 0, ef = 0;
    std::vector<float> q;
    std::vector<int32_t> ids;
    std::vector<float> dis;
    int slot0 = -1;
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
    int err = GSX_OK;
    std::string msg;
    Clock::time_point t_submit, t_done;
};

struct Group {
    std::vector<Request *> reqs;  // consecutive slot ranges starting at slot0
    int slot0 = -1, nq = 0;
    std::atomic<bool> done{false};
    std::condition_variable *wake = nullptr;
};

}  // namespace

struct gsx_server {
    gsx_searcher *s = nullptr;
    int capacity = 0, kcap = 0, efcap = 0, nstreams = 0, d = 0, max_group = 0;
    std::vector<cudaStream_t> streams;
    std::vector<Group *> running;  // per stream
    DevBuf dq, dids, ddis, dk, def, dstatus, dorder, dcnt;
    std::vector<std::unique_ptr<SpillTables>> spill;  // per stream: visited-set spill tables of the group's warps
    float *hq = nullptr;
    int32_t *hids = nullptr, *hk = nullptr, *hef = nullptr, *horder = nullptr, *hstatus = nullptr;
    float *hdis = nullptr;
    Ranges ranges;
    std::mutex mu;
    std::condition_variable cv;       // dispatcher wake-ups
    std::condition_variable done_cv;  // waiters
    std::deque<Request *> queue;
    std::map<uint64_t, Request *> reqs;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread th;
    int64_t completed_queries = 0;
    int dispatch_error = GSX_OK;
    std::string dispatch_msg;
};

namespace {

// Host callback at the end of a group's stream work: no CUDA calls, only a flag and a wake-up.
void CUDART_CB on_group_done(void *p) {
    auto *g = static_cast<Group *>(p);
    g->done.store(true, std::memory_order_release);
    g->wake->notify_one();
}

// Copies a finished group's results to its requests and frees their slots (mu held).
void finish_group(gsx_server *sv, Group *g) {
    for (Request *r : g->reqs) {
        for (int i = 0; i < r->nq; ++i) {
            const int slot = r->slot0 + i;
            std::memcpy(&r->ids[(size_t)i * r->k], sv->hids + (size_t)slot * sv->kcap, (size_t)r->k * 4);
            std::memcpy(&r->dis[(size_t)i * r->k], sv->hdis + (size_t)slot * sv->kcap, (size_t)r->k * 4);
            if (sv->hstatus[slot] != 0) {
                // visited table overflow: answer this query exactly on the searcher's own stream
                int rc = server_resolve_one(sv->s, &r->q[(size_t)i * sv->d], r->k, r->ef, &r->ids[(size_t)i * r->k],
                                            &r->dis[(size_t)i * r->k]);
                if (rc != GSX_OK) {
                    r->err = rc;
                    r->msg = gsx_last_error();
                }
            }
        }
        r->state = r->err == GSX_OK ? 2 : 3;
        r->t_done = Clock::now();
        sv->completed_queries += r->nq;
    }
    sv->ranges.give(g->slot0, g->nq);
    delete g;
}

// Enqueues one admitted group on stream `si` (mu NOT held; slots already reserved).
int launch_group(gsx_server *sv, Group *g, int si) {
    cudaStream_t st = sv->streams[si];
    const int d = sv->d;
    int n = 0, kmax = 1, efmax = 1;
    int32_t *order = sv->horder + (size_t)si * sv->capacity;
    for (Request *r : g->reqs) {
        std::memcpy(sv->hq + (size_t)r->slot0 * d, r->q.data(), (size_t)r->nq * d * 4);
        for (int i = 0; i < r->nq; ++i) {
            sv->hk[r->slot0 + i] = r->k;
            sv->hef[r->slot0 + i] = r->ef;
            order[n++] = r->slot0 + i;
        }
        kmax = std::max(kmax, r->k);
        efmax = std::max(efmax, r->ef);
    }
    const size_t o = (size_t)g->slot0;
    GSX_CUDA(cudaMemcpyAsync(sv->dq.as<float>() + o * d, sv->hq + o * d, (size_t)n * d * 4, cudaMemcpyHostToDevice, st));
    GSX_CUDA(cudaMemcpyAsync(sv->dk.as<int32_t>() + o, sv->hk + o, (size_t)n * 4, cudaMemcpyHostToDevice, st));
    GSX_CUDA(cudaMemcpyAsync(sv->def.as<int32_t>() + o, sv->hef + o, (size_t)n * 4, cudaMemcpyHostToDevice, st));
    // longest searches first (largest ef, then k), so that the group's tail is short
    std::stable_sort(order, order + n, [&](int32_t a, int32_t b) {
        return sv->hef[a] != sv->hef[b] ? sv->hef[a] > sv->hef[b] : sv->hk[a] > sv->hk[b];
    });
    int32_t *dorder = sv->dorder.as<int32_t>() + (size_t)si * sv->capacity;
    GSX_CUDA(cudaMemcpyAsync(dorder, order, (size_t)n * 4, cudaMemcpyHostToDevice, st));
    unsigned *cnt = sv->dcnt.as<unsigned>() + 2 * si;
    GSX_CUDA(cudaMemsetAsync(cnt, 0, 8, st));
    LaunchCfg cfg;
    int sbits = 0;
    int rc = server_make_cfg(sv->s, kmax, efmax, n, &cfg, &sbits);
    if (rc) return rc;
    BatchView bv{};
    bv.queries = sv->dq.as<float>();
    bv.nq = n;
    bv.k = kmax;
    bv.ef = efmax;
    bv.k_per = sv->dk.as<int32_t>();
    bv.ef_per = sv->def.as<int32_t>();
    bv.order = dorder;
    bv.out_stride = sv->kcap;
    bv.out_ids = sv->dids.as<int32_t>();
    bv.out_dis = sv->ddis.as<float>();
    bv.status = sv->dstatus.as<int32_t>();
    bv.counter = cnt;
    bv.overflow = cnt + 1;
    bv.gtab_shift = visited_id_bits(sv->s->ix.N);
    if ((rc = sv->spill[si]->ensure((size_t)cfg.max_blocks * cfg.warps_per_block, sbits, bv.gtab_shift, st, &bv.gtab,
                                    &bv.gtab_epoch)))
        return rc;
    bv.gtab_bits = sbits;
    GSX_CUDA(launch_search(sv->s->ix, bv, cfg, st));
    GSX_CUDA(cudaMemcpyAsync(sv->hids + o * sv->kcap, sv->dids.as<int32_t>() + o * sv->kcap, (size_t)n * sv->kcap * 4,
                             cudaMemcpyDeviceToHost, st));
    GSX_CUDA(cudaMemcpyAsync(sv->hdis + o * sv->kcap, sv->ddis.as<float>() + o * sv->kcap, (size_t)n * sv->kcap * 4,
                             cudaMemcpyDeviceToHost, st));
    GSX_CUDA(cudaMemcpyAsync(sv->hstatus + o, sv->dstatus.as<int32_t>() + o, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    GSX_CUDA(cudaLaunchHostFunc(st, on_group_done, g));
    return GSX_OK;
}

void dispatcher(gsx_server *sv) {
    cudaSetDevice(sv->s->device);
    std::unique_lock<std::mutex> lk(sv->mu);
    while (true) {
        bool progressed = false;
        // 1. retire finished groups
        for (int si = 0; si < sv->nstreams; ++si) {
            Group *g = sv->running[si];
            if (g && g->done.load(std::memory_order_acquire)) {
                sv->running[si] = nullptr;
                finish_group(sv, g);
                progressed = true;
            }
        }
        if (progressed) sv->done_cv.notify_all();
        if (sv->stop && sv->queue.empty()) {
            bool any = false;
            for (Group *g : sv->running) any |= g != nullptr;
            if (!any) break;
        }
        // 2. admit the oldest queued requests into a free stream
        int si = -1;
        for (int i = 0; i < sv->nstreams; ++i)
            if (!sv->running[i]) { si = i; break; }
        if (si >= 0 && !sv->queue.empty()) {
            auto *g = new Group;
            g->wake = &sv->cv;
            // groups stay small enough that slots cycle quickly (a group's slots free only when its
            // slowest query is done) and fit the largest free range; FIFO, no overtaking
            const int room = std::min(sv->max_group, sv->ranges.largest());
            int gq = 0;
            size_t nr = 0;
            for (Request *r : sv->queue) {
                if (gq + r->nq > room && (gq > 0 || r->nq > sv->ranges.largest())) break;
                gq += r->nq;
                ++nr;
                if (gq >= room) break;
            }
            if (nr > 0) {
                g->slot0 = sv->ranges.take(gq);
                g->nq = gq;
                int s0 = g->slot0;
                for (size_t i = 0; i < nr; ++i) {
                    Request *r = sv->queue.front();
                    sv->queue.pop_front();
                    r->slot0 = s0;
                    r->state = 1;
                    s0 += r->nq;
                    g->reqs.push_back(r);
                }
            }
            if (!g->reqs.empty()) {
                sv->running[si] = g;
                lk.unlock();
                const int rc = launch_group(sv, g, si);
                lk.lock();
                if (rc != GSX_OK) {
                    // nothing was left queued on the stream for this group that can complete it
                    cudaStreamSynchronize(sv->streams[si]);
                    sv->running[si] = nullptr;
                    sv->ranges.give(g->slot0, g->nq);
                    for (Request *r : g->reqs) {
                        r->state = 3;
                        r->err = rc;
                        r->msg = gsx_last_error();
                        r->t_done = Clock::now();
                    }
                    delete g;
                    sv->done_cv.notify_all();
                }
                continue;
            }
            delete g;
        }
        // 3. sleep until a submission or a completion wakes us (bounded, in case a wake-up races
        //    with this check)
        sv->cv.wait_for(lk, std::chrono::microseconds(500));
    }
}

}  // namespace

extern "C" {

int gsx_server_create(gsx_searcher *s, int32_t max_queries_in_flight, int32_t kmax, int32_t efmax, int32_t streams,
                      gsx_server **out) {
    try {
        if (!s || !out) return fail(GSX_ERR_INVALID, "null argument");
        if (!s->has_data) return fail(GSX_ERR_STATE, "server before set_data");
        if (max_queries_in_flight <= 0 || kmax <= 0 || efmax <= 0 || streams <= 0 || streams > 32)
            return fail(GSX_ERR_INVALID, "bad server arguments");
        int rc;
        GSX_CUDA(cudaSetDevice(s->device));
        auto *sv = new gsx_server;
        sv->s = s;
        sv->kcap = kmax;
        sv->efcap = efmax;
        sv->nstreams = streams;
        sv->d = s->ix.d;
        // memory-based admission: the slot arena is sized so that it takes at most half of the free
        // device memory
        const size_t per_slot = (size_t)sv->d * 4 + (size_t)kmax * 8 + 16 + (size_t)streams * 4;
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        size_t cap = (size_t)max_queries_in_flight;
        if (per_slot * cap > free_b / 2) cap = std::max<size_t>(1, free_b / 2 / per_slot);
        sv->capacity = (int)cap;
        sv->max_group = std::max(256, sv->capacity / (2 * streams));
        auto bad = [&](int code) {
            gsx_server_destroy(sv);
            return code;
        };
        if ((rc = sv->dq.ensure(cap * sv->d * 4)) || (rc = sv->dids.ensure(cap * kmax * 4)) ||
            (rc = sv->ddis.ensure(cap * kmax * 4)) || (rc = sv->dk.ensure(cap * 4)) || (rc = sv->def.ensure(cap * 4)) ||
            (rc = sv->dstatus.ensure(cap * 4)) || (rc = sv->dorder.ensure(cap * 4 * streams)) ||
            (rc = sv->dcnt.ensure(64 * streams)))
            return bad(rc);
        auto pin = [&](void **p, size_t bytes) { return cudaHostAlloc(p, bytes, cudaHostAllocDefault) == cudaSuccess; };
        if (!pin((void **)&sv->hq, cap * sv->d * 4) || !pin((void **)&sv->hids, cap * kmax * 4) ||
            !pin((void **)&sv->hdis, cap * kmax * 4) || !pin((void **)&sv->hk, cap * 4) || !pin((void **)&sv->hef, cap * 4) ||
            !pin((void **)&sv->horder, cap * 4 * streams) || !pin((void **)&sv->hstatus, cap * 4))
            return bad(fail(GSX_ERR_NOMEM, "pinned host allocation failed"));
        sv->streams.resize(streams, nullptr);
        sv->running.assign(streams, nullptr);
        for (int i = 0; i < streams; ++i) sv->spill.emplace_back(new SpillTables);
        for (auto &st : sv->streams) {
            cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
            if (e != cudaSuccess) return bad(cuda_fail(e, "cudaStreamCreate"));
        }
        sv->ranges.init(sv->capacity);
        sv->th = std::thread(dispatcher, sv);
        *out = sv;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_server_create")
}

int gsx_server_capacity(const gsx_server *sv, int32_t *slots) {
    try {
        if (!sv || !slots) return fail(GSX_ERR_INVALID, "null argument");
        *slots = sv->capacity;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_server_capacity")
}

int gsx_server_submit(gsx_server *sv, const float *queries, int32_t nq, int32_t k, int32_t ef, uint64_t *ticket) {
    try {
        if (!sv || !queries || !ticket) return fail(GSX_ERR_INVALID, "null argument");
        if (nq <= 0 || k <= 0 || ef <= 0) return fail(GSX_ERR_INVALID, "nq, k and ef must be positive");
        if (k > sv->kcap || ef > sv->efcap) return fail(GSX_ERR_INVALID, "k or ef above the server's limits");
        if (nq > sv->capacity) return fail(GSX_ERR_NOMEM, "request of %d queries exceeds the %d admitted slots", nq, sv->capacity);
        auto *r = new Request;
        r->nq = nq;
        r->k = k;
        r->ef = ef;
        r->q.assign(queries, queries + (size_t)nq * sv->d);
        r->ids.assign((size_t)nq * k, -1);
        r->dis.assign((size_t)nq * k, 0.0f);
        r->t_submit = Clock::now();
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            if (sv->stop) {
                delete r;
                return fail(GSX_ERR_STATE, "server is stopping");
            }
            r->ticket = sv->next_ticket++;
            sv->reqs[r->ticket] = r;
            sv->queue.push_back(r);
        }
        sv->cv.notify_one();
        *ticket = r->ticket;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_server_submit")
}

int gsx_server_wait(gsx_server *sv, uint64_t ticket, int32_t timeout_ms, int32_t *ids, float *dis, double *latency_ms) {
    try {
        if (!sv) return fail(GSX_ERR_INVALID, "null server");
        std::unique_lock<std::mutex> lk(sv->mu);
        auto it = sv->reqs.find(ticket);
        if (it == sv->reqs.end()) return fail(GSX_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
        Request *r = it->second;
        const auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
        while (r->state < 2) {
            if (sv->done_cv.wait_until(lk, deadline) == std::cv_status::timeout && r->state < 2)
                return fail(GSX_ERR_TIMEOUT, "request %llu not finished within %d ms", (unsigned long long)ticket, timeout_ms);
        }
        sv->reqs.erase(it);
        lk.unlock();
        std::unique_ptr<Request> own(r);
        if (r->state == 3) return fail(r->err, "%s", r->msg.c_str());
        if (ids) std::memcpy(ids, r->ids.data(), r->ids.size() * 4);
        if (dis) std::memcpy(dis, r->dis.data(), r->dis.size() * 4);
        if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_server_wait")
}

int gsx_server_stats(gsx_server *sv, int64_t *completed_queries, int32_t *queued_requests, int32_t *running_groups) {
    try {
        if (!sv) return fail(GSX_ERR_INVALID, "null server");
        std::lock_guard<std::mutex> lk(sv->mu);
        if (completed_queries) *completed_queries = sv->completed_queries;
        if (queued_requests) *queued_requests = (int32_t)sv->queue.size();
        if (running_groups) {
            int n = 0;
            for (Group *g : sv->running) n += g != nullptr;
            *running_groups = n;
        }
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_server_stats")
}

int gsx_server_drive_poisson(gsx_server *sv, const float *queries, int32_t nq_pool, int32_t n_requests,
                             double request_rate, int32_t size_min, int32_t size_max, const int32_t *ks, int32_t nk,
                             const int32_t *efs, int32_t nef, uint64_t seed, double *latency_ms, int32_t *sizes,
                             double *wall_s) {
    try {
        if (!sv || !queries || !ks || !efs || !latency_ms || nk <= 0 || nef <= 0 || n_requests <= 0 || request_rate <= 0 ||
            size_min <= 0 || size_max < size_min || size_max > nq_pool || size_max > sv->capacity)
            return fail(GSX_ERR_INVALID, "bad load-driver arguments");
        const int d = sv->d;
        std::mt19937_64 rng(seed);
        std::exponential_distribution<double> gap(request_rate);
        std::uniform_real_distribution<double> u01(0.0, 1.0);
        std::vector<double> at(n_requests);
        std::vector<int32_t> sz(n_requests), kk(n_requests), ee(n_requests), off(n_requests);
        double t = 0.0;
        int64_t pos = 0;
        const double lmin = std::log((double)size_min), lmax = std::log((double)size_max + 1.0);
        for (int i = 0; i < n_requests; ++i) {
            t += gap(rng);
            at[i] = t;
            sz[i] = std::min(size_max, (int32_t)std::floor(std::exp(lmin + (lmax - lmin) * u01(rng))));
            kk[i] = ks[rng() % (uint64_t)nk];
            ee[i] = efs[rng() % (uint64_t)nef];
            if (pos + sz[i] > nq_pool) pos = 0;
            off[i] = (int32_t)pos;
            pos += sz[i];
        }
        std::vector<uint64_t> tickets(n_requests, 0);
        std::atomic<int> submitted{0};
        std::atomic<int> err{GSX_OK};
        const auto t0 = Clock::now();
        std::thread producer([&] {
            for (int i = 0; i < n_requests; ++i) {
                const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(at[i]));
                // sleep most of the gap, then spin (bounded by the due time) for sub-millisecond precision
                if (due - Clock::now() > std::chrono::microseconds(200))
                    std::this_thread::sleep_until(due - std::chrono::microseconds(100));
                while (Clock::now() < due) {
                }
                uint64_t tk = 0;
                const int rc = gsx_server_submit(sv, queries + (size_t)off[i] * d, sz[i], kk[i], ee[i], &tk);
                if (rc != GSX_OK) {
                    err.store(rc);
                    break;
                }
                tickets[i] = tk;
                submitted.store(i + 1, std::memory_order_release);
            }
        });
        int rc = GSX_OK;
        for (int i = 0; i < n_requests && rc == GSX_OK; ++i) {
            while (submitted.load(std::memory_order_acquire) <= i) {
                if (err.load() != GSX_OK) break;
                std::this_thread::sleep_for(std::chrono::microseconds(20));
            }
            if (err.load() != GSX_OK) {
                rc = err.load();
                break;
            }
            rc = gsx_server_wait(sv, tickets[i], 120000, nullptr, nullptr, &latency_ms[i]);
            if (sizes) sizes[i] = sz[i];
        }
        producer.join();
        if (wall_s) *wall_s = std::chrono::duration<double>(Clock::now() - t0).count();
        if (rc == GSX_OK && err.load() != GSX_OK) rc = err.load();
        return rc;
    } GSX_ABI_GUARD("gsx_server_drive_poisson")
}

void gsx_server_destroy(gsx_server *sv) {
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv.notify_all();
    if (sv->th.joinable()) sv->th.join();
    cudaSetDevice(sv->s->device);
    for (auto st : sv->streams)
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    for (auto &kv : sv->reqs) delete kv.second;
    for (void *p : {(void *)sv->hq, (void *)sv->hids, (void *)sv->hdis, (void *)sv->hk, (void *)sv->hef,
                    (void *)sv->horder, (void *)sv->hstatus})
        if (p) cudaFreeHost(p);
    delete sv;
}

}  // extern "C"
