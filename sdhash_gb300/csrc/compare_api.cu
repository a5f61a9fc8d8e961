// compare_api.cu -- digest sets on the device and the comparison entry
// points of the C ABI (include/sdbf_gb300.h).
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include <atomic>

#include "ctx_internal.h"
#include "matrix_plan.h"

static std::atomic<uint64_t> g_set_serial{1};

uint64_t next_set_serial() { return g_set_serial.fetch_add(1); }

// -------------------------------------------------------------- comparison
extern "C" int sdbfg_set_upload(sdbfg_ctx* c, const sdbfg_digest_desc* ds, uint32_t n, sdbfg_set** out) {
    if (!c || !out || (n && !ds)) return SDBFG_ERR_ARG;
    *out = nullptr;
    CUDA_TRY(c, cudaSetDevice(c->device));
    auto* s = new sdbfg_set();
    s->ctx = c;
    s->n = n;
    s->serial = next_set_serial();
    uint64_t total = 0;
    std::vector<CmpDigest> dig(n);
    for (uint32_t i = 0; i < n; i++) {
        if (ds[i].bf_count == 0 || !ds[i].filters) {
            delete s;
            return fail(c, SDBFG_ERR_ARG, "digest %u has no filters", i);
        }
        dig[i] = {(uint32_t)total, ds[i].bf_count};
        total += ds[i].bf_count;
    }
    if (total >= (1ull << 32)) {
        delete s;
        return fail(c, SDBFG_ERR_ARG, "set too large");
    }
    s->total_filters = total;
    std::vector<uint32_t> meta(total);
    std::vector<uint8_t> filt(total * 256);
    s->names.resize(n);
    s->fast.assign(n, 0);
    s->bf_count.resize(n);
    s->last_elem.resize(n);
    s->orig_size.resize(n);
    s->max_elem.resize(n);
    s->last_count.resize(n);
    s->dd_block.resize(n);
    s->first.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        const sdbfg_digest_desc& d = ds[i];
        s->names[i] = d.name ? d.name : "";
        s->bf_count[i] = d.bf_count;
        s->orig_size[i] = d.orig_size;
        s->max_elem[i] = d.max_elem;
        s->last_count[i] = d.elem_counts ? 0 : d.last_count;
        s->dd_block[i] = d.elem_counts ? d.dd_block_size : 0;
        s->first[i] = dig[i].first;
        memcpy(&filt[(uint64_t)dig[i].first * 256], d.filters, (uint64_t)d.bf_count * 256);
        for (uint32_t f = 0; f < d.bf_count; f++) {
            // get_elem_count (sdbf_class.cc:406-415)
            uint32_t e = d.elem_counts ? d.elem_counts[f] : (f + 1 < d.bf_count ? d.max_elem : d.last_count);
            uint32_t h = 0;
            const uint8_t* p = d.filters + (uint64_t)f * 256;
            for (int b = 0; b < 256; b += 8) {
                uint64_t w;
                memcpy(&w, p + b, 8);
                h += (uint32_t)__builtin_popcountll(w);
            }
            meta[dig[i].first + f] = (h << 16) | (e & 0xFFFFu);
            if (f + 1 == d.bf_count) s->last_elem[i] = e;
        }
    }
    if (s->d_filters.ensure(std::max<uint64_t>(1, total) * 256) || s->d_meta.ensure(std::max<uint64_t>(1, total) * 4) ||
        s->d_digests.ensure(std::max<uint32_t>(1, n) * sizeof(CmpDigest))) {
        s->d_filters.release();
        s->d_meta.release();
        s->d_digests.release();
        delete s;
        return fail(c, SDBFG_ERR_NOMEM, "set upload: out of device memory");
    }
    cudaMemcpy(s->d_filters.p, filt.data(), total * 256, cudaMemcpyHostToDevice);
    cudaMemcpy(s->d_meta.p, meta.data(), total * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(s->d_digests.p, dig.data(), n * sizeof(CmpDigest), cudaMemcpyHostToDevice);
    *out = s;
    return SDBFG_OK;
}

static void drop_plans(sdbfg_ctx* c, uint64_t serial) {
    auto& plans = c->plans;
    for (size_t k = 0; k < plans.size();) {
        if (plans[k]->serial_a == serial || plans[k]->serial_b == serial) {
            delete plans[k];
            plans.erase(plans.begin() + k);
        } else {
            k++;
        }
    }
}

extern "C" int sdbfg_set_fast(sdbfg_ctx* c, sdbfg_set* s, uint32_t first, uint32_t count) {
    if (!c || !s || first > s->n || count > s->n - first) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (!count) return SDBFG_OK;
    TIMED_LAUNCH(c, "k_fold", launch_fold(s->d_filters.as<uint32_t>(), s->d_meta.as<uint32_t>(),
                                          s->d_digests.as<CmpDigest>(), first, count, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    for (uint32_t i = first; i < first + count; i++) s->fast[i] = 1;
    drop_plans(c, s->serial);  // group units are formed per fast mode
    return SDBFG_OK;
}

extern "C" void sdbfg_set_free(sdbfg_set* s) {
    if (!s) return;
    cudaSetDevice(s->ctx->device);
    drop_plans(s->ctx, s->serial);
    s->d_filters.release();
    s->d_meta.release();
    s->d_digests.release();
    delete s;
}

extern "C" uint32_t sdbfg_set_size(const sdbfg_set* s) { return s ? s->n : 0; }

// Orientation of a pair: sdbf_score's swap rule (sdbf_core.cc:351-359).
static CmpPair orient(const sdbfg_set* a, uint32_t i, const sdbfg_set* b, uint32_t j) {
    const uint32_t n1 = a->bf_count[i], n2 = b->bf_count[j];
    const bool swap = n1 > n2 || (n1 == n2 && (a->last_elem[i] > b->last_elem[j] ||
                                               strcmp(a->names[i].c_str(), b->names[j].c_str()) > 0));
    if (swap) return CmpPair{j, i, n2, 1u | 0u};  // ref from b (side 1), tgt from a (side 0)
    return CmpPair{i, j, n1, 2u};                  // ref from a (side 0), tgt from b (side 1)
}

static int run_pairs(sdbfg_ctx* c, const sdbfg_set* a, const sdbfg_set* b, const std::vector<CmpPair>& pairs,
                     int32_t* out) {
    cudaStream_t st = c->stream;
    CUDA_TRY(c, c->d_pairs.ensure(std::max<size_t>(1, pairs.size()) * sizeof(CmpPair)));
    CUDA_TRY(c, c->d_scores.ensure(std::max<size_t>(1, pairs.size()) * 4));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_pairs.p, pairs.data(), pairs.size() * sizeof(CmpPair), cudaMemcpyHostToDevice,
                                st));
    CmpParams P{};
    P.filters[0] = a->d_filters.as<uint32_t>();
    P.meta[0] = a->d_meta.as<uint32_t>();
    P.digests[0] = a->d_digests.as<CmpDigest>();
    P.filters[1] = b->d_filters.as<uint32_t>();
    P.meta[1] = b->d_meta.as<uint32_t>();
    P.digests[1] = b->d_digests.as<CmpDigest>();
    P.pairs = c->d_pairs.as<CmpPair>();
    P.npairs = pairs.size();
    P.scores = c->d_scores.as<int32_t>();
    P.cutoffs = c->d_cut.as<uint16_t>();
    P.cutoffs64 = c->d_cut64.as<uint16_t>();
    const uint32_t grid = (uint32_t)std::min<uint64_t>(pairs.size(), (uint64_t)c->sms * 16);
    TIMED_LAUNCH(c, "k_compare_pairs", launch_compare_pairs(P, std::max(1u, grid), st));
    CUDA_TRY(c, cudaMemcpyAsync(out, c->d_scores.p, pairs.size() * 4, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaStreamSynchronize(st));
    return SDBFG_OK;
}

extern "C" int sdbfg_score_pairs(sdbfg_ctx* c, const sdbfg_set* a, const sdbfg_set* b, const uint32_t* ia,
                                 const uint32_t* ib, uint64_t npairs, int32_t* out) {
    if (!c || !a || !b || (npairs && (!ia || !ib || !out))) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    for (uint64_t base = 0; base < npairs; base += kPairsPerLaunch) {
        const uint64_t m = std::min<uint64_t>(kPairsPerLaunch, npairs - base);
        std::vector<CmpPair> pairs(m);
        for (uint64_t k = 0; k < m; k++) {
            const uint32_t i = ia[base + k], j = ib[base + k];
            if (i >= a->n || j >= b->n) return fail(c, SDBFG_ERR_ARG, "pair %llu out of range", (unsigned long long)k);
            pairs[k] = orient(a, i, b, j);
        }
        int rc = run_pairs(c, a, b, pairs, out + base);
        if (rc) return rc;
    }
    return SDBFG_OK;
}

// ------------------------------------------------------- matrix engine
// Orientation of pair (x of set a, y of set b) called as sdbf_score(x, y):
// true when y becomes the reference (the swap rule, sdbf_core.cc:351-359).
static bool swaps(const sdbfg_set* a, uint32_t x, const sdbfg_set* b, uint32_t y) {
    const uint32_t n1 = a->bf_count[x], n2 = b->bf_count[y];
    return n1 > n2 ||
           (n1 == n2 && (a->last_elem[x] > b->last_elem[y] || strcmp(a->names[x].c_str(), b->names[y].c_str()) > 0));
}

static MatPlan* find_plan(sdbfg_ctx* c, uint64_t sa, uint64_t sb, uint32_t mode) {
    static uint64_t tick = 0;
    for (MatPlan* p : c->plans)
        if (p->serial_a == sa && p->serial_b == sb && p->mode == mode && p->variant == c->mat_variant &&
            p->unit_work == c->mat_unit_work) {
            p->last_use = ++tick;
            return p;
        }
    return nullptr;
}

static int upload_plan(sdbfg_ctx* c, MatPlan* p, UnitBuilder& ub, const std::vector<uint32_t>& targets) {
    const std::vector<MatUnit> units = ub.sorted_units();
    p->nunits = (uint32_t)units.size();
    p->nsplit = (uint32_t)ub.split.size();
    p->filter_pairs = ub.filter_pairs;
    CUDA_TRY(c, p->d_units.ensure(std::max<size_t>(1, units.size()) * sizeof(MatUnit)));
    CUDA_TRY(c, p->d_targets.ensure(std::max<size_t>(1, targets.size()) * 4));
    CUDA_TRY(c, p->d_split.ensure(std::max<size_t>(1, ub.split.size()) * sizeof(MatSplit)));
    CUDA_TRY(c, p->d_refs.ensure(std::max<size_t>(1, ub.refs.size()) * 4));
    if (!ub.refs.empty())
        CUDA_TRY(c, cudaMemcpyAsync(p->d_refs.p, ub.refs.data(), ub.refs.size() * 4, cudaMemcpyHostToDevice,
                                    c->stream));
    CUDA_TRY(c, p->d_slots.ensure(std::max<uint64_t>(1, ub.slots) * 8));
    CUDA_TRY(c, p->d_counter.ensure(64));
    cudaStream_t st = c->stream;
    if (!units.empty())
        CUDA_TRY(c, cudaMemcpyAsync(p->d_units.p, units.data(), units.size() * sizeof(MatUnit),
                                    cudaMemcpyHostToDevice, st));
    if (!targets.empty())
        CUDA_TRY(c, cudaMemcpyAsync(p->d_targets.p, targets.data(), targets.size() * 4, cudaMemcpyHostToDevice, st));
    if (!ub.split.empty())
        CUDA_TRY(c, cudaMemcpyAsync(p->d_split.p, ub.split.data(), ub.split.size() * sizeof(MatSplit),
                                    cudaMemcpyHostToDevice, st));
    CUDA_TRY(c, cudaStreamSynchronize(st));  // host vectors go out of scope
    return SDBFG_OK;
}

// All pairs i<j of one set.  Digests sorted by filter count: a digest is the
// reference for every digest with more filters (a suffix of the sorted
// order, shared by all) and for the equal-count digests the swap rule gives
// it (explicit lists appended to the target list).
static int build_plan_all(sdbfg_ctx* c, const sdbfg_set* s, MatPlan* p) {
    const uint32_t n = s->n;
    std::vector<uint32_t> sorted(n);
    std::iota(sorted.begin(), sorted.end(), 0u);
    std::stable_sort(sorted.begin(), sorted.end(),
                     [&](uint32_t x, uint32_t y) { return s->bf_count[x] < s->bf_count[y]; });
    std::vector<uint32_t> targets(sorted);
    uint64_t sum = 0, sum2 = 0;
    for (uint32_t i = 0; i < n; i++) {
        sum += s->bf_count[i];
        sum2 += (uint64_t)s->bf_count[i] * s->bf_count[i];
    }
    const uint64_t ctas = (uint64_t)c->sms * matrix_ctas_per_sm(c->mat_variant);
    UnitBuilder ub(effective_unit_budget(c->mat_unit_work, (sum * sum - sum2) / 2, ctas),
                   (uint32_t)kMatVariantTable[c->mat_variant].rows);
    const auto nf = [&](uint32_t e) { return s->bf_count[targets[e]]; };
    const auto id = [&](uint32_t e) { return targets[e]; };
    const auto nf_ref = [&](uint32_t d) { return s->bf_count[d]; };
    uint32_t g0 = 0;
    while (g0 < n) {
        uint32_t g1 = g0;
        while (g1 < n && s->bf_count[sorted[g1]] == s->bf_count[sorted[g0]]) g1++;
        // every digest of the group is the reference of the whole suffix
        const std::vector<uint32_t> ids(sorted.begin() + g0, sorted.begin() + g1);
        ub.add_shared(ids, nf_ref, [&](uint32_t d) { return (uint32_t)s->fast[d]; }, 0u, g1, n, nf, id);
        // and of the equal-count digests the swap rule gives it
        for (uint32_t k = g0; k < g1; k++) {
            const uint32_t a = sorted[k];
            const uint32_t tie0 = (uint32_t)targets.size();
            for (uint32_t m = g0; m < g1; m++) {
                const uint32_t b = sorted[m];
                if (b == a) continue;
                const uint32_t i = std::min(a, b), j = std::max(a, b);
                const uint32_t ref = swaps(s, i, s, j) ? j : i;
                if (ref == a) targets.push_back(b);
            }
            ub.add(a, s->bf_count[a], 0u, tie0, (uint32_t)targets.size(), nf, id);
        }
        g0 = g1;
    }
    p->nscores = (uint64_t)n * (n - 1) / 2;
    return upload_plan(c, p, ub, targets);
}

// Every query of set q against every target of set t (sdbf_score(q_i, t_j)).
static int build_plan_cross(sdbfg_ctx* c, const sdbfg_set* q, const sdbfg_set* t, MatPlan* p) {
    if ((uint64_t)q->n * t->n + q->n + t->n >= (1ull << 32))
        return fail(c, SDBFG_ERR_ARG, "compare_to: too many pairs for one plan");
    const uint64_t ctas = (uint64_t)c->sms * matrix_ctas_per_sm(c->mat_variant);
    UnitBuilder ub(effective_unit_budget(c->mat_unit_work, (uint64_t)q->total_filters * t->total_filters, ctas),
                   (uint32_t)kMatVariantTable[c->mat_variant].rows);
    std::vector<uint32_t> targets;
    build_cross_units(
        ub, targets, q->n, t->n, [&](uint32_t i, uint32_t j) { return swaps(q, i, t, j); },
        [&](uint32_t i) { return q->bf_count[i]; }, [&](uint32_t j) { return t->bf_count[j]; },
        [&](uint32_t i) { return (uint32_t)q->fast[i]; }, [&](uint32_t j) { return (uint32_t)t->fast[j]; });
    p->nscores = (uint64_t)q->n * t->n;
    return upload_plan(c, p, ub, targets);
}

static int get_plan(sdbfg_ctx* c, const sdbfg_set* a, const sdbfg_set* b, uint32_t mode, MatPlan** out) {
    const uint64_t sb = b ? b->serial : 0;
    MatPlan* p = find_plan(c, a->serial, sb, mode);
    if (!p) {
        if (c->plans.size() >= 8) {  // drop the least recently used plan
            auto it = std::min_element(c->plans.begin(), c->plans.end(),
                                       [](MatPlan* x, MatPlan* y) { return x->last_use < y->last_use; });
            delete *it;
            c->plans.erase(it);
        }
        p = new MatPlan();
        p->serial_a = a->serial;
        p->serial_b = sb;
        p->mode = mode;
        p->variant = c->mat_variant;
        p->unit_work = c->mat_unit_work;
        const int rc = mode == kMatModeAll ? build_plan_all(c, a, p) : build_plan_cross(c, a, b, p);
        if (rc) {
            delete p;
            return rc;
        }
        c->plans.push_back(p);
        find_plan(c, a->serial, sb, mode);
    }
    *out = p;
    return SDBFG_OK;
}

static MatParams plan_params(sdbfg_ctx* c, const MatPlan* p, const sdbfg_set* a, const sdbfg_set* b,
                             int32_t* scores) {
    MatParams P{};
    const sdbfg_set* s1 = b ? b : a;
    P.filters[0] = a->d_filters.as<uint32_t>();
    P.meta[0] = a->d_meta.as<uint32_t>();
    P.digests[0] = a->d_digests.as<CmpDigest>();
    P.filters[1] = s1->d_filters.as<uint32_t>();
    P.meta[1] = s1->d_meta.as<uint32_t>();
    P.digests[1] = s1->d_digests.as<CmpDigest>();
    P.units = p->d_units.as<MatUnit>();
    P.nunits = p->nunits;
    P.next_unit = p->d_counter.as<uint32_t>();
    P.targets = p->d_targets.as<uint32_t>();
    P.refs = p->d_refs.as<uint32_t>();
    P.split = p->d_split.as<MatSplit>();
    P.nsplit = p->nsplit;
    P.slots = p->d_slots.as<double>();
    P.scores = scores;
    P.mode = p->mode;
    P.n = p->mode == kMatModeAll ? a->n : b->n;
    P.cutoffs = c->d_cut.as<uint16_t>();
    P.cutoffs64 = c->d_cut64.as<uint16_t>();
    P.error = p->d_counter.as<uint32_t>() + 1;
    P.phase = c->profile ? c->d_mphase.as<unsigned long long>() : nullptr;
    return P;
}

static int enqueue_plan(sdbfg_ctx* c, const MatPlan* p, const MatParams& P, cudaStream_t st) {
    CUDA_TRY(c, cudaMemsetAsync(p->d_counter.p, 0, 8, st));  // work counter, error flag
    const uint32_t grid = (uint32_t)(c->sms * matrix_ctas_per_sm(p->variant));
    TIMED_LAUNCH_ON(c, "k_matrix", st, launch_matrix(P, p->variant, std::max(1u, std::min(grid, P.nunits)), st));
    if (P.nsplit) TIMED_LAUNCH_ON(c, "k_matrix_finalize", st, launch_matrix_finalize(P, st));
    return SDBFG_OK;
}

// Runs a plan on the context stream, replaying its CUDA graph when the
// output array is the one it was captured with.
static int run_plan(sdbfg_ctx* c, MatPlan* p, const sdbfg_set* a, const sdbfg_set* b, int32_t* dev_scores) {
    cudaStream_t st = c->stream;
    const MatParams P = plan_params(c, p, a, b, dev_scores);
    matrix_ctas_per_sm(p->variant);  // sets the kernel's attributes outside any capture
    if (!c->mat_graphs || c->profile) return enqueue_plan(c, p, P, st);
    if (p->graph && p->graph_out == dev_scores) {
        CUDA_TRY(c, cudaGraphLaunch(p->graph, st));
        c->launches += 1 + (P.nsplit ? 1 : 0);
        return SDBFG_OK;
    }
    if (p->graph) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    // capture on a private stream so a caller's stream in capture mode is not disturbed
    cudaStream_t cs;
    CUDA_TRY(c, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = SDBFG_OK;
    if (e == cudaSuccess) {
        rc = enqueue_plan(c, p, P, cs);
        e = cudaStreamEndCapture(cs, &g);
    }
    cudaStreamDestroy(cs);
    if (rc) return rc;
    c->launches -= 1 + (P.nsplit ? 1 : 0);  // counted when the graph runs
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(c, SDBFG_ERR_CUDA, "comparison graph: %s", cudaGetErrorString(e));
    p->graph_out = dev_scores;
    CUDA_TRY(c, cudaGraphLaunch(p->graph, st));
    c->launches += 1 + (P.nsplit ? 1 : 0);
    return SDBFG_OK;
}

// waits for the plan's launches and reports a bounded wait that gave up
static int check_plan_error(sdbfg_ctx* c, const MatPlan* p) {
    uint32_t err = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&err, p->d_counter.as<uint32_t>() + 1, 4, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (err) return fail(c, SDBFG_ERR_CUDA, "comparison kernel: %u CTAs gave up waiting for the tensor cores", err);
    return SDBFG_OK;
}

extern "C" int sdbfg_compare_all_device(sdbfg_ctx* c, const sdbfg_set* s, int32_t* dev_scores) {
    if (!c || !s || (!dev_scores && s->n > 1)) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (s->n < 2) return SDBFG_OK;
    MatPlan* p;
    int rc = get_plan(c, s, nullptr, kMatModeAll, &p);
    if (rc) return rc;
    return run_plan(c, p, s, nullptr, dev_scores);
}

extern "C" int sdbfg_compare_to_device(sdbfg_ctx* c, const sdbfg_set* q, const sdbfg_set* t, int32_t* dev_scores) {
    if (!c || !q || !t || (!dev_scores && q->n && t->n)) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (!q->n || !t->n) return SDBFG_OK;
    MatPlan* p;
    int rc = get_plan(c, q, t, kMatModeCross, &p);
    if (rc) return rc;
    return run_plan(c, p, q, t, dev_scores);
}

extern "C" int sdbfg_compare_all(sdbfg_ctx* c, const sdbfg_set* s, int32_t* out) {
    if (!c || !s || (!out && s->n > 1)) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (s->n < 2) return SDBFG_OK;
    MatPlan* p;
    int rc = get_plan(c, s, nullptr, kMatModeAll, &p);
    if (rc) return rc;
    CUDA_TRY(c, c->d_scores.ensure(p->nscores * 4));
    rc = run_plan(c, p, s, nullptr, c->d_scores.as<int32_t>());
    if (rc) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(out, c->d_scores.p, p->nscores * 4, cudaMemcpyDeviceToHost, c->stream));
    return check_plan_error(c, p);
}

extern "C" int sdbfg_compare_to(sdbfg_ctx* c, const sdbfg_set* q, const sdbfg_set* t, int32_t* out) {
    if (!c || !q || !t || (!out && q->n && t->n)) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (!q->n || !t->n) return SDBFG_OK;
    MatPlan* p;
    int rc = get_plan(c, q, t, kMatModeCross, &p);
    if (rc) return rc;
    CUDA_TRY(c, c->d_scores.ensure(p->nscores * 4));
    rc = run_plan(c, p, q, t, c->d_scores.as<int32_t>());
    if (rc) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(out, c->d_scores.p, p->nscores * 4, cudaMemcpyDeviceToHost, c->stream));
    return check_plan_error(c, p);
}

// scores (already queued into c->d_scores) -> matches on the host
static int collect_matches(sdbfg_ctx* c, uint64_t nscores, uint32_t mode, uint64_t dim, int32_t threshold,
                           sdbfg_match* out, uint64_t cap, uint64_t* count) {
    cudaStream_t st = c->stream;
    const uint64_t nb = (nscores + kMatchBlockScores - 1) / kMatchBlockScores;
    CUDA_TRY(c, c->d_match_counts.ensure(std::max<uint64_t>(1, nb) * 4));
    CUDA_TRY(c, c->d_match_offs.ensure((nb + 1) * 8));
    const int32_t* sc = c->d_scores.as<int32_t>();
    TIMED_LAUNCH_ON(c, "k_match_count", st, launch_match_count(sc, nscores, threshold, c->d_match_counts.as<uint32_t>(), st));
    TIMED_LAUNCH_ON(c, "k_match_scan", st, launch_match_scan(c->d_match_counts.as<uint32_t>(), nb,
                                                             c->d_match_offs.as<uint64_t>(), st));
    uint64_t total = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&total, c->d_match_offs.as<uint64_t>() + nb, 8, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaStreamSynchronize(st));
    *count = total;
    if (total > cap) return fail(c, SDBFG_ERR_CAPACITY, "%llu matches, room for %llu", (unsigned long long)total,
                                 (unsigned long long)cap);
    if (!total) return SDBFG_OK;
    CUDA_TRY(c, c->d_matches.ensure(total * sizeof(sdbfg_match)));
    TIMED_LAUNCH_ON(c, "k_match_write", st, launch_match_write(sc, nscores, threshold, c->d_match_offs.as<uint64_t>(),
                                                               mode, dim, c->d_matches.as<uint32_t>(), total, st));
    CUDA_TRY(c, cudaMemcpyAsync(out, c->d_matches.p, total * sizeof(sdbfg_match), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaStreamSynchronize(st));
    return SDBFG_OK;
}

extern "C" int sdbfg_compare_all_matches(sdbfg_ctx* c, const sdbfg_set* s, int32_t threshold, sdbfg_match* out,
                                         uint64_t cap, uint64_t* count) {
    if (!c || !s || !count || (cap && !out)) return SDBFG_ERR_ARG;
    *count = 0;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (s->n < 2) return SDBFG_OK;
    MatPlan* p;
    int rc = get_plan(c, s, nullptr, kMatModeAll, &p);
    if (rc) return rc;
    CUDA_TRY(c, c->d_scores.ensure(p->nscores * 4));
    rc = run_plan(c, p, s, nullptr, c->d_scores.as<int32_t>());
    if (rc) return rc;
    if ((rc = check_plan_error(c, p))) return rc;
    return collect_matches(c, p->nscores, kMatModeAll, s->n, threshold, out, cap, count);
}

extern "C" int sdbfg_compare_to_matches(sdbfg_ctx* c, const sdbfg_set* q, const sdbfg_set* t, int32_t threshold,
                                        sdbfg_match* out, uint64_t cap, uint64_t* count) {
    if (!c || !q || !t || !count || (cap && !out)) return SDBFG_ERR_ARG;
    *count = 0;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (!q->n || !t->n) return SDBFG_OK;
    MatPlan* p;
    int rc = get_plan(c, q, t, kMatModeCross, &p);
    if (rc) return rc;
    CUDA_TRY(c, c->d_scores.ensure(p->nscores * 4));
    rc = run_plan(c, p, q, t, c->d_scores.as<int32_t>());
    if (rc) return rc;
    if ((rc = check_plan_error(c, p))) return rc;
    return collect_matches(c, p->nscores, kMatModeCross, t->n, threshold, out, cap, count);
}

extern "C" int sdbfg_ctx_set_compare_tuning(sdbfg_ctx* c, int variant, uint64_t unit_work, int use_graphs) {
    if (!c || variant < 0 || variant >= kMatVariants || unit_work == 0) return SDBFG_ERR_ARG;
    c->mat_variant = variant;
    c->mat_unit_work = unit_work;
    c->mat_graphs = use_graphs != 0;
    return SDBFG_OK;
}

extern "C" int sdbfg_ctx_get_compare_tuning(const sdbfg_ctx* c, int* variant, uint64_t* unit_work) {
    if (!c) return SDBFG_ERR_ARG;
    if (variant) *variant = c->mat_variant;
    if (unit_work) *unit_work = c->mat_unit_work;
    return SDBFG_OK;
}

extern "C" uint64_t sdbfg_compare_filter_pairs(sdbfg_ctx* c, const sdbfg_set* a, const sdbfg_set* b) {
    if (!c || !a) return 0;
    MatPlan* p;
    if (get_plan(c, a, b, b ? kMatModeCross : kMatModeAll, &p)) return 0;
    return p->filter_pairs;
}

// Times every kernel variant and unit budget on a sample of the plan's units
// (every k-th unit, about `sample_pairs` filter pairs) and keeps the fastest.
extern "C" int sdbfg_compare_autotune(sdbfg_ctx* c, const sdbfg_set* a, const sdbfg_set* b, uint64_t sample_pairs,
                                      int* out_variant, uint64_t* out_unit_work, double* out_rate) {
    if (!c || !a) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    const uint32_t mode = b ? kMatModeCross : kMatModeAll;
    const uint64_t budgets[3] = {1ull << 20, 1ull << 22, 1ull << 24};
    const int saved_v = c->mat_variant;
    const uint64_t saved_w = c->mat_unit_work;
    int best_v = saved_v;
    uint64_t best_w = saved_w;
    double best_rate = -1;
    cudaEvent_t e0, e1;
    CUDA_TRY(c, cudaEventCreate(&e0));
    CUDA_TRY(c, cudaEventCreate(&e1));
    for (uint64_t w : budgets) {
        for (int v = 0; v < kMatVariants; v++) {
            c->mat_variant = v;
            c->mat_unit_work = w;
            MatPlan* p;
            int rc = get_plan(c, a, b, mode, &p);
            if (rc) return rc;
            // sampled unit list: every k-th unit (the plan is sorted largest first)
            std::vector<MatUnit> units(p->nunits);
            CUDA_TRY(c, cudaMemcpy(units.data(), p->d_units.p, units.size() * sizeof(MatUnit), cudaMemcpyDeviceToHost));
            const uint64_t avg = std::max<uint64_t>(1, p->filter_pairs / std::max<uint32_t>(1, p->nunits));
            const uint64_t want = std::max<uint64_t>(1, sample_pairs / avg);
            const uint64_t step = std::max<uint64_t>(1, units.size() / want);
            std::vector<MatUnit> sample;
            for (uint64_t k = 0; k < units.size(); k += step)
                if (!(units[k].flags & kUnitSplit)) sample.push_back(units[k]);
            if (sample.empty()) continue;
            uint64_t pairs = 0;
            std::vector<uint32_t> tl;  // target list for work counting
            DevBuf d_sample;
            CUDA_TRY(c, d_sample.ensure(sample.size() * sizeof(MatUnit)));
            CUDA_TRY(c, cudaMemcpy(d_sample.p, sample.data(), sample.size() * sizeof(MatUnit), cudaMemcpyHostToDevice));
            CUDA_TRY(c, c->d_scores.ensure(p->nscores * 4));
            MatParams P = plan_params(c, p, a, b, c->d_scores.as<int32_t>());
            P.units = d_sample.as<MatUnit>();
            P.nunits = (uint32_t)sample.size();
            P.nsplit = 0;
            {
                std::vector<uint32_t> targets;
                // count filter pairs of the sample from the target list on the host
                const sdbfg_set* ts_all = b ? b : a;
                size_t tn = 0;
                for (const MatUnit& u : sample) tn = std::max<size_t>(tn, u.t1);
                targets.resize(tn);
                if (tn) CUDA_TRY(c, cudaMemcpy(targets.data(), p->d_targets.p, tn * 4, cudaMemcpyDeviceToHost));
                for (const MatUnit& u : sample) {
                    const sdbfg_set* rset = (u.flags & kUnitRefSide1) ? ts_all : a;
                    const sdbfg_set* tset = (u.flags & kUnitTgtSide1) ? ts_all : a;
                    (void)rset;
                    for (uint32_t e = u.t0; e < u.t1; e++) pairs += (uint64_t)(u.r1 - u.r0) * tset->bf_count[targets[e]];
                }
            }
            cudaStream_t st = c->stream;
            float best_ms = 1e30f;
            for (int rep = 0; rep < 2; rep++) {
                CUDA_TRY(c, cudaMemsetAsync(p->d_counter.p, 0, 8, st));
                CUDA_TRY(c, cudaEventRecord(e0, st));
                const uint32_t grid = (uint32_t)(c->sms * matrix_ctas_per_sm(v));
                CUDA_TRY(c, launch_matrix(P, v, std::max(1u, std::min(grid, P.nunits)), st));
                CUDA_TRY(c, cudaEventRecord(e1, st));
                CUDA_TRY(c, cudaEventSynchronize(e1));
                float ms = 0;
                CUDA_TRY(c, cudaEventElapsedTime(&ms, e0, e1));
                best_ms = std::min(best_ms, ms);
            }
            d_sample.release();
            const double rate = pairs / (best_ms * 1e-3);
            if (rate > best_rate) {
                best_rate = rate;
                best_v = v;
                best_w = w;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->mat_variant = best_v;
    c->mat_unit_work = best_w;
    (void)saved_v;
    (void)saved_w;
    if (out_variant) *out_variant = best_v;
    if (out_unit_work) *out_unit_work = best_w;
    if (out_rate) *out_rate = best_rate;
    return SDBFG_OK;
}
