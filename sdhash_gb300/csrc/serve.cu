// serve.cu -- a query-serving loop over a device-resident reference set.
//
// The reference compares query digests against a target set with one
// OpenMP loop per call (sdbf_set::compare_to, sdbf/sdbf_set.cc:318-346);
// each call is independent.  Here a worker thread keeps the target set
// resident and serves a stream of query digests with continuous batching:
//
//   * requests queue on the host as they arrive (sdbfg_server_submit);
//   * a fixed number of batch slots, each with its own CUDA stream, pinned
//     staging and device buffers sized at creation (no allocation while
//     serving), run concurrently on the GPU;
//   * when a slot is free, the worker admits queued requests in arrival
//     order while their filters fit the slot's device memory (admission by
//     memory), stages them, builds the batch's work units (every query
//     against every target, orientation by the swap rule) and queues
//     upload -> k_matrix -> finalize -> scores download on the slot stream;
//   * requests that arrive while batches are on the GPU wait only for the
//     next free slot, so their work overlaps with the batches in flight.
//
// A query's scores do not depend on its batch: every digest pair is scored
// by the same exact kernel path whatever else shares the launch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "ctx_internal.h"
#include "matrix_plan.h"

namespace {

uint64_t now_ns() {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Request {
    uint64_t tag = 0;
    std::string name;
    uint32_t nf = 0, last = 0;
    std::vector<uint8_t> filters;   // nf * 256
    std::vector<uint32_t> meta;     // (hamming << 16) | element count
    uint64_t submit_ns = 0, start_ns = 0;
};

struct Done {
    sdbfg_server_result r;
    std::vector<int32_t> scores;
};

}  // namespace

struct sdbfg_server {
    sdbfg_ctx* ctx = nullptr;
    const sdbfg_set* refs = nullptr;
    sdbfg_server_config cfg{};
    uint32_t slot_filters = 0;  // admission limit per batch (device memory)
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv, cv_done;
    bool stop = false;
    std::string err;
    std::deque<Request> pending;
    std::deque<Done> done;
    std::atomic<uint64_t> launches{0}, batches{0}, served{0};
    struct Slot {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        bool busy = false;
        std::vector<Request> batch;
        uint32_t nunits = 0, nsplit = 0;
        HostBuf h_filters, h_meta, h_dig, h_units, h_targets, h_refs, h_split, h_scores;
        DevBuf d_filters, d_meta, d_dig, d_units, d_targets, d_refs, d_split, d_slots, d_counter, d_scores;
        uint64_t cap_units = 0, cap_targets = 0, cap_refs = 0, cap_split = 0, cap_slots = 0;
    };
    std::vector<Slot> slots;
};

static bool server_swaps(const Request& q, const sdbfg_set* t, uint32_t j) {
    const uint32_t n1 = q.nf, n2 = t->bf_count[j];
    return n1 > n2 || (n1 == n2 && (q.last > t->last_elem[j] || strcmp(q.name.c_str(), t->names[j].c_str()) > 0));
}

// Grows a slot buffer outside the serving hot path (first batches only).
static cudaError_t grow(DevBuf& d, HostBuf* h, uint64_t& cap, uint64_t need, size_t elem) {
    if (need <= cap) return cudaSuccess;
    const uint64_t want = std::max<uint64_t>(need, cap * 2);
    cudaError_t e = d.ensure(want * elem);
    if (e == cudaSuccess && h) e = h->ensure(want * elem);
    if (e == cudaSuccess) cap = want;
    return e;
}

// Stage and launch one batch on slot S.  Returns a CUDA error or success.
static cudaError_t launch_batch(sdbfg_server* sv, sdbfg_server::Slot& S) {
    const sdbfg_set* T = sv->refs;
    const uint32_t nq = (uint32_t)S.batch.size(), nt = T->n;
    // query filters / meta / digest table
    uint64_t tot = 0;
    CmpDigest* dig = S.h_dig.as<CmpDigest>();
    for (uint32_t i = 0; i < nq; i++) {
        const Request& r = S.batch[i];
        memcpy(S.h_filters.as<uint8_t>() + tot * 256, r.filters.data(), (size_t)r.nf * 256);
        memcpy(S.h_meta.as<uint32_t>() + tot, r.meta.data(), (size_t)r.nf * 4);
        dig[i] = CmpDigest{(uint32_t)tot, r.nf};
        tot += r.nf;
    }
    // work units: every query against every target, orientation by the swap rule
    const uint64_t ctas = (uint64_t)sv->ctx->sms * matrix_ctas_per_sm(sv->ctx->mat_variant);
    UnitBuilder ub(effective_unit_budget(sv->ctx->mat_unit_work, tot * T->total_filters, ctas),
                   (uint32_t)kMatVariantTable[sv->ctx->mat_variant].rows);
    std::vector<uint32_t> targets;
    build_cross_units(
        ub, targets, nq, nt, [&](uint32_t i, uint32_t j) { return server_swaps(S.batch[i], T, j); },
        [&](uint32_t i) { return S.batch[i].nf; }, [&](uint32_t j) { return T->bf_count[j]; },
        [](uint32_t) { return 0u; }, [&](uint32_t j) { return (uint32_t)T->fast[j]; });
    const std::vector<MatUnit> units = ub.sorted_units();
    cudaError_t e;
    if ((e = grow(S.d_units, &S.h_units, S.cap_units, units.size() + 1, sizeof(MatUnit)))) return e;
    if ((e = grow(S.d_targets, &S.h_targets, S.cap_targets, targets.size() + 1, 4))) return e;
    if ((e = grow(S.d_split, &S.h_split, S.cap_split, ub.split.size() + 1, sizeof(MatSplit)))) return e;
    if ((e = grow(S.d_refs, &S.h_refs, S.cap_refs, ub.refs.size() + 1, 4))) return e;
    memcpy(S.h_refs.p, ub.refs.data(), ub.refs.size() * 4);
    if ((e = grow(S.d_slots, nullptr, S.cap_slots, ub.slots + 1, 8))) return e;
    memcpy(S.h_units.p, units.data(), units.size() * sizeof(MatUnit));
    memcpy(S.h_targets.p, targets.data(), targets.size() * 4);
    memcpy(S.h_split.p, ub.split.data(), ub.split.size() * sizeof(MatSplit));
    S.nunits = (uint32_t)units.size();
    S.nsplit = (uint32_t)ub.split.size();
    cudaStream_t st = S.st;
    if ((e = cudaMemcpyAsync(S.d_filters.p, S.h_filters.p, tot * 256, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(S.d_meta.p, S.h_meta.p, tot * 4, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(S.d_dig.p, S.h_dig.p, nq * sizeof(CmpDigest), cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(S.d_units.p, S.h_units.p, units.size() * sizeof(MatUnit), cudaMemcpyHostToDevice, st)))
        return e;
    if ((e = cudaMemcpyAsync(S.d_targets.p, S.h_targets.p, targets.size() * 4, cudaMemcpyHostToDevice, st))) return e;
    if (!ub.refs.empty() &&
        (e = cudaMemcpyAsync(S.d_refs.p, S.h_refs.p, ub.refs.size() * 4, cudaMemcpyHostToDevice, st)))
        return e;
    if (S.nsplit &&
        (e = cudaMemcpyAsync(S.d_split.p, S.h_split.p, S.nsplit * sizeof(MatSplit), cudaMemcpyHostToDevice, st)))
        return e;
    if ((e = cudaMemsetAsync(S.d_counter.p, 0, 8, st))) return e;  // work counter, error flag
    MatParams P{};
    P.filters[0] = S.d_filters.as<uint32_t>();
    P.meta[0] = S.d_meta.as<uint32_t>();
    P.digests[0] = S.d_dig.as<CmpDigest>();
    P.filters[1] = T->d_filters.as<uint32_t>();
    P.meta[1] = T->d_meta.as<uint32_t>();
    P.digests[1] = T->d_digests.as<CmpDigest>();
    P.units = S.d_units.as<MatUnit>();
    P.nunits = S.nunits;
    P.next_unit = S.d_counter.as<uint32_t>();
    P.targets = S.d_targets.as<uint32_t>();
    P.refs = S.d_refs.as<uint32_t>();
    P.split = S.d_split.as<MatSplit>();
    P.nsplit = S.nsplit;
    P.slots = S.d_slots.as<double>();
    P.scores = S.d_scores.as<int32_t>();
    P.mode = kMatModeCross;
    P.n = nt;
    P.cutoffs = sv->ctx->d_cut.as<uint16_t>();
    P.cutoffs64 = sv->ctx->d_cut64.as<uint16_t>();
    P.error = S.d_counter.as<uint32_t>() + 1;
    const uint32_t grid = (uint32_t)std::min<uint64_t>(ctas, std::max(1u, S.nunits));
    if ((e = launch_matrix(P, sv->ctx->mat_variant, grid, st))) return e;
    if ((e = launch_matrix_finalize(P, st))) return e;
    sv->launches += 1 + (S.nsplit ? 1 : 0);
    if ((e = cudaMemcpyAsync(S.h_scores.p, S.d_scores.p, (size_t)nq * nt * 4, cudaMemcpyDeviceToHost, st))) return e;
    return cudaEventRecord(S.ev, st);
}

static void finish_batch(sdbfg_server* sv, sdbfg_server::Slot& S) {
    const uint32_t nt = sv->refs->n;
    const uint64_t t = now_ns();
    const int32_t* sc = S.h_scores.as<int32_t>();
    std::vector<Done> out(S.batch.size());
    for (size_t i = 0; i < S.batch.size(); i++) {
        Done& d = out[i];
        const int32_t* row = sc + i * nt;
        d.scores.assign(row, row + nt);
        d.r.tag = S.batch[i].tag;
        d.r.status = 0;
        d.r.best_score = -1;
        d.r.best_target = 0;
        d.r.matches = 0;
        for (uint32_t j = 0; j < nt; j++) {
            if (row[j] > d.r.best_score) {
                d.r.best_score = row[j];
                d.r.best_target = j;
            }
            d.r.matches += row[j] >= sv->cfg.threshold;
        }
        d.r.batch_queries = (uint32_t)S.batch.size();
        d.r.submit_ns = S.batch[i].submit_ns;
        d.r.start_ns = S.batch[i].start_ns;
        d.r.done_ns = t;
    }
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        for (Done& d : out) sv->done.push_back(std::move(d));
    }
    sv->served += S.batch.size();
    sv->batches += 1;
    S.batch.clear();
    S.busy = false;
    sv->cv_done.notify_all();
}

static void worker_loop(sdbfg_server* sv) {
    cudaSetDevice(sv->ctx->device);
    for (;;) {
        // retire finished batches
        bool any_busy = false;
        for (auto& S : sv->slots) {
            if (!S.busy) continue;
            const cudaError_t q = cudaEventQuery(S.ev);
            if (q == cudaSuccess) {
                finish_batch(sv, S);
            } else if (q != cudaErrorNotReady) {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->err = cudaGetErrorString(q);
                sv->stop = true;
            } else {
                any_busy = true;
            }
        }
        // admit queued requests into free slots
        for (auto& S : sv->slots) {
            if (S.busy) continue;
            {
                std::unique_lock<std::mutex> lk(sv->mu);
                if (sv->pending.empty()) break;
                uint64_t f = 0;
                const uint64_t t = now_ns();
                const uint64_t tf = sv->refs->total_filters;
                while (!sv->pending.empty() && S.batch.size() < sv->cfg.max_batch_queries &&
                       (S.batch.empty() || (f + sv->pending.front().nf <= sv->slot_filters &&
                                            (f + sv->pending.front().nf) * tf <= sv->cfg.max_batch_pairs))) {
                    f += sv->pending.front().nf;
                    S.batch.push_back(std::move(sv->pending.front()));
                    S.batch.back().start_ns = t;
                    sv->pending.pop_front();
                }
            }
            const cudaError_t e = launch_batch(sv, S);
            if (e != cudaSuccess) {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->err = cudaGetErrorString(e);
                sv->stop = true;
                break;
            }
            S.busy = true;
            any_busy = true;
        }
        std::unique_lock<std::mutex> lk(sv->mu);
        if (!sv->err.empty()) break;
        if (sv->stop && sv->pending.empty() && !any_busy) break;
        if (!any_busy && sv->pending.empty()) {
            sv->cv.wait_for(lk, std::chrono::milliseconds(2));
        } else if (any_busy) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    }
    // drain whatever is still on the GPU
    for (auto& S : sv->slots)
        if (S.busy) {
            cudaEventSynchronize(S.ev);
            finish_batch(sv, S);
        }
}

extern "C" int sdbfg_server_create(sdbfg_ctx* c, const sdbfg_set* refs, const sdbfg_server_config* cfg,
                                   sdbfg_server** out) {
    if (!c || !refs || !out || refs->n == 0) return SDBFG_ERR_ARG;
    *out = nullptr;
    CUDA_TRY(c, cudaSetDevice(c->device));
    auto* sv = new sdbfg_server();
    sv->ctx = c;
    sv->refs = refs;
    sdbfg_server_config d{3, 256, 256ull << 20, 1, 0, 1ull << 31};
    if (cfg) d = *cfg;
    if (d.max_batch_pairs == 0) d.max_batch_pairs = 1ull << 31;
    if (d.slots == 0 || d.slots > 8 || d.max_batch_queries == 0 || d.memory_budget < (1ull << 20)) {
        delete sv;
        return fail(c, SDBFG_ERR_ARG, "server config out of range");
    }
    sv->cfg = d;
    // device bytes per admitted filter: filter, meta, split slots against
    // every target; plus per query one row of scores
    const uint64_t per_filter = 256 + 4 + 8ull * refs->n;
    sv->slot_filters = (uint32_t)std::max<uint64_t>(4096, d.memory_budget / d.slots / per_filter);
    sv->slots.resize(d.slots);
    matrix_ctas_per_sm(c->mat_variant);
    for (auto& S : sv->slots) {
        cudaError_t e = cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S.ev, cudaEventDisableTiming);
        const uint64_t nf = sv->slot_filters, nq = d.max_batch_queries;
        for (auto [dv, hv, bytes] : {std::tuple<DevBuf*, HostBuf*, uint64_t>{&S.d_filters, &S.h_filters, nf * 256},
                                     {&S.d_meta, &S.h_meta, nf * 4},
                                     {&S.d_dig, &S.h_dig, nq * sizeof(CmpDigest)},
                                     {&S.d_scores, &S.h_scores, nq * refs->n * 4}}) {
            if (e == cudaSuccess) e = dv->ensure(bytes);
            if (e == cudaSuccess) e = hv->ensure(bytes);
        }
        if (e == cudaSuccess) e = S.d_counter.ensure(64);
        if (e == cudaSuccess) e = grow(S.d_units, &S.h_units, S.cap_units, 1 << 16, sizeof(MatUnit));
        if (e == cudaSuccess)
            e = grow(S.d_targets, &S.h_targets, S.cap_targets, (uint64_t)nq * refs->n + nq + refs->n + 1, 4);
        if (e == cudaSuccess) e = grow(S.d_refs, &S.h_refs, S.cap_refs, (uint64_t)nq + refs->n + 1, 4);
        if (e == cudaSuccess) e = grow(S.d_split, &S.h_split, S.cap_split, (uint64_t)nq * refs->n + 1, sizeof(MatSplit));
        if (e == cudaSuccess) e = grow(S.d_slots, nullptr, S.cap_slots, (uint64_t)nf * refs->n + 1, 8);
        if (e != cudaSuccess) {
            sdbfg_server_destroy(sv);
            return fail(c, e == cudaErrorMemoryAllocation ? SDBFG_ERR_NOMEM : SDBFG_ERR_CUDA, "server slots: %s",
                        cudaGetErrorString(e));
        }
    }
    sv->worker = std::thread(worker_loop, sv);
    *out = sv;
    return SDBFG_OK;
}

extern "C" int sdbfg_server_submit(sdbfg_server* sv, const sdbfg_digest_desc* q, uint64_t tag) {
    if (!sv || !q || q->bf_count == 0 || !q->filters) return SDBFG_ERR_ARG;
    if (q->bf_count > sv->slot_filters) return SDBFG_ERR_CAPACITY;
    Request r;
    r.tag = tag;
    r.name = q->name ? q->name : "";
    r.nf = q->bf_count;
    r.filters.assign(q->filters, q->filters + (size_t)q->bf_count * 256);
    r.meta.resize(q->bf_count);
    for (uint32_t f = 0; f < q->bf_count; f++) {
        // get_elem_count (sdbf_class.cc:406-415) and hamming (sdbf_class.cc:388-401)
        const uint32_t e = q->elem_counts ? q->elem_counts[f] : (f + 1 < q->bf_count ? q->max_elem : q->last_count);
        uint32_t h = 0;
        for (int b = 0; b < 256; b += 8) {
            uint64_t w;
            memcpy(&w, q->filters + (size_t)f * 256 + b, 8);
            h += (uint32_t)__builtin_popcountll(w);
        }
        r.meta[f] = (h << 16) | (e & 0xFFFFu);
        if (f + 1 == q->bf_count) r.last = e;
    }
    r.submit_ns = now_ns();
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stop) return SDBFG_ERR_ARG;
        sv->pending.push_back(std::move(r));
    }
    sv->cv.notify_one();
    return SDBFG_OK;
}

extern "C" int sdbfg_server_poll(sdbfg_server* sv, sdbfg_server_result* out, int32_t* scores, uint32_t max,
                                 uint32_t* n, int timeout_ms) {
    if (!sv || !out || !n) return SDBFG_ERR_ARG;
    *n = 0;
    std::unique_lock<std::mutex> lk(sv->mu);
    if (sv->done.empty() && timeout_ms != 0) {
        const auto pred = [&] { return !sv->done.empty() || !sv->err.empty(); };
        if (timeout_ms < 0) sv->cv_done.wait(lk, pred);
        else sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred);
    }
    const uint32_t nt = sv->refs->n;
    while (*n < max && !sv->done.empty()) {
        Done& d = sv->done.front();
        out[*n] = d.r;
        if (scores) memcpy(scores + (size_t)*n * nt, d.scores.data(), (size_t)nt * 4);
        sv->done.pop_front();
        (*n)++;
    }
    if (!sv->err.empty()) return fail(sv->ctx, SDBFG_ERR_CUDA, "server: %s", sv->err.c_str());
    return SDBFG_OK;
}

extern "C" int sdbfg_server_stats(const sdbfg_server* sv, uint64_t* pending, uint64_t* served, uint64_t* batches,
                                  uint64_t* launches) {
    if (!sv) return SDBFG_ERR_ARG;
    auto* m = const_cast<sdbfg_server*>(sv);
    if (pending) {
        std::lock_guard<std::mutex> lk(m->mu);
        *pending = m->pending.size();
    }
    if (served) *served = sv->served.load();
    if (batches) *batches = sv->batches.load();
    if (launches) *launches = sv->launches.load();
    return SDBFG_OK;
}

extern "C" void sdbfg_server_destroy(sdbfg_server* sv) {
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    cudaSetDevice(sv->ctx->device);
    for (auto& S : sv->slots) {
        for (DevBuf* b : {&S.d_filters, &S.d_meta, &S.d_dig, &S.d_units, &S.d_targets, &S.d_refs, &S.d_split,
                          &S.d_slots, &S.d_counter, &S.d_scores})
            b->release();
        for (HostBuf* b : {&S.h_filters, &S.h_meta, &S.h_dig, &S.h_units, &S.h_targets, &S.h_refs, &S.h_split,
                           &S.h_scores})
            b->release();
        if (S.st) cudaStreamDestroy(S.st);
        if (S.ev) cudaEventDestroy(S.ev);
    }
    delete sv;
}
