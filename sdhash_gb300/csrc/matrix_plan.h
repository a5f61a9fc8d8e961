// matrix_plan.h -- work-unit construction for the batched comparison
// engine (k_matrix), shared by the set comparison entry points and the
// serving loop.  Host code only.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

#include "compare_kernels.h"

namespace sdbfg {

// Accumulates work units.  A reference digest with at most `max_rows`
// filters goes into a group unit (alone or with other digests that share
// its target list, see add_group); a larger one gets multi-pass units, and a
// single pair larger than the budget is row-split.  Target runs are cut at
// the work budget (filter pairs) and at kMatMaxTargets targets.
struct UnitBuilder {
    std::vector<MatUnit> units;
    std::vector<uint64_t> work;  // per unit, for the largest-first order
    std::vector<MatSplit> split;
    std::vector<uint32_t> refs;  // reference digest ids of group units
    uint64_t slots = 0;
    uint64_t budget;
    uint32_t max_rows;
    uint64_t filter_pairs = 0;
    UnitBuilder(uint64_t w, uint32_t rows) : budget(std::max<uint64_t>(w, 1)), max_rows(rows) {}

    // target run [t0, t1) of the target list for `rows` reference rows
    template <class NF, class EMIT>
    void cut_runs(uint32_t rows, uint32_t t0, uint32_t t1, NF nf, EMIT emit) {
        uint32_t start = t0;
        uint64_t acc = 0;
        for (uint32_t e = t0; e < t1; e++) {
            const uint64_t w = (uint64_t)rows * nf(e);
            if (e > start && (acc + w > budget || e - start >= kMatMaxTargets)) {
                emit(start, e, acc);
                start = e;
                acc = 0;
            }
            acc += w;
        }
        if (t1 > start) emit(start, t1, acc);
    }

    // digests ids[0..n) (side flags) all against targets [t0, t1); their
    // filters together must fit max_rows
    template <class NF>
    void add_group(const uint32_t* ids, uint32_t n, uint32_t rows, uint32_t flags, uint32_t t0, uint32_t t1, NF nf) {
        const uint32_t pos = (uint32_t)refs.size();
        refs.insert(refs.end(), ids, ids + n);
        cut_runs(rows, t0, t1, nf, [&](uint32_t a, uint32_t b, uint64_t acc) {
            units.push_back(MatUnit{pos, 0, rows, a, b, flags | kUnitGroup, 0, n});
            work.push_back(acc + (uint64_t)(b - a) * rows * 4);
            filter_pairs += acc;
        });
    }

    // one reference digest against targets [t0, t1)
    template <class NF, class ID>
    void add(uint32_t ref, uint32_t nref, uint32_t flags, uint32_t t0, uint32_t t1, NF nf, ID id) {
        if (t1 <= t0) return;
        if (nref <= max_rows) {
            add_group(&ref, 1, nref, flags, t0, t1, nf);
            return;
        }
        uint32_t start = t0;
        uint64_t acc = 0;
        auto flush = [&](uint32_t end) {
            if (end > start) {
                units.push_back(MatUnit{ref, 0, nref, start, end, flags, 0, 1});
                work.push_back(acc + (uint64_t)(end - start) * nref * 4);
            }
            start = end;
            acc = 0;
        };
        for (uint32_t e = t0; e < t1; e++) {
            const uint64_t w = (uint64_t)nref * nf(e);
            filter_pairs += w;
            if (w > budget) {  // one pair larger than a unit: split the reference's rows
                flush(e);
                const uint32_t rows = (uint32_t)std::max<uint64_t>(128, budget / nf(e) / 128 * 128);
                const uint32_t si = (uint32_t)split.size();
                split.push_back(MatSplit{ref, id(e), flags & (kUnitRefSide1 | kUnitTgtSide1), 0, slots});
                slots += nref;
                for (uint32_t r = 0; r < nref; r += rows) {
                    const uint32_t r1 = std::min(nref, r + rows);
                    units.push_back(MatUnit{ref, r, r1, e, e + 1, flags | kUnitSplit, si, 1});
                    work.push_back((uint64_t)(r1 - r) * nf(e));
                }
                start = e + 1;
                continue;
            }
            if (e > start && (acc + w > budget || e - start >= kMatMaxTargets)) flush(e);
            acc += w;
        }
        flush(t1);
    }

    // digests ids[0..n) with counts nf_ref, all sharing the target run
    // [t0, t1): packed into groups of at most max_rows filters (those with
    // more filters go through add)
    // (a group holds digests of one fast mode only: key(d) separates them)
    template <class NFR, class KEY, class NF, class ID>
    void add_shared(const std::vector<uint32_t>& ids, NFR nf_ref, KEY key, uint32_t flags, uint32_t t0, uint32_t t1,
                    NF nf, ID id) {
        if (t1 <= t0) return;
        std::vector<uint32_t> cur;
        uint32_t rows = 0, cur_key = 0;
        auto flush = [&]() {
            if (!cur.empty()) add_group(cur.data(), (uint32_t)cur.size(), rows, flags, t0, t1, nf);
            cur.clear();
            rows = 0;
        };
        for (uint32_t d : ids) {
            const uint32_t n = nf_ref(d);
            if (n > max_rows) {
                add(d, n, flags, t0, t1, nf, id);
                continue;
            }
            const uint32_t k = key(d);
            if (rows + n > max_rows || (!cur.empty() && k != cur_key)) flush();
            cur.push_back(d);
            cur_key = k;
            rows += n;
        }
        flush();
    }

    // units largest first (LPT order for the persistent CTAs)
    std::vector<MatUnit> sorted_units() const {
        std::vector<uint32_t> order(units.size());
        for (uint32_t k = 0; k < order.size(); k++) order[k] = k;
        std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return work[x] > work[y]; });
        std::vector<MatUnit> out(units.size());
        for (size_t k = 0; k < order.size(); k++) out[k] = units[order[k]];
        return out;
    }
};

// Units of a query x target job: query digest i (side 0) against target
// digest j (side 1), scored as sdbf_score(query i, target j); swaps(i, j) is
// the swap rule (true: the target is the reference).  The target list holds
// one run of all targets (shared by every query that is the reference
// against all of them), one run of all queries (likewise for targets), then
// explicit runs for the rest.
template <class SW, class NQ, class NT, class KQ, class KT>
void build_cross_units(UnitBuilder& ub, std::vector<uint32_t>& targets, uint32_t nq, uint32_t nt, SW swaps,
                       NQ nf_q, NT nf_t, KQ key_q, KT key_t) {
    std::vector<uint8_t> sw((size_t)nq * nt);
    std::vector<uint32_t> cnt_q(nq, 0), cnt_t(nt, 0);
    for (uint32_t i = 0; i < nq; i++)
        for (uint32_t j = 0; j < nt; j++) {
            const bool x = swaps(i, j);
            sw[(size_t)i * nt + j] = x;
            if (x) cnt_t[j]++;
            else cnt_q[i]++;
        }
    targets.clear();
    for (uint32_t j = 0; j < nt; j++) targets.push_back(j);  // [0, nt): all targets
    for (uint32_t i = 0; i < nq; i++) targets.push_back(i);  // [nt, nt+nq): all queries
    const auto tid_ = [&](uint32_t e) { return targets[e]; };
    const auto nft = [&](uint32_t e) { return nf_t(targets[e]); };
    const auto nfq = [&](uint32_t e) { return nf_q(targets[e]); };
    std::vector<uint32_t> full_q, full_t;
    for (uint32_t i = 0; i < nq; i++)
        if (cnt_q[i] == nt) full_q.push_back(i);
    for (uint32_t j = 0; j < nt; j++)
        if (cnt_t[j] == nq) full_t.push_back(j);
    ub.add_shared(full_q, nf_q, key_q, kUnitTgtSide1, 0, nt, nft, tid_);
    ub.add_shared(full_t, nf_t, key_t, kUnitRefSide1, nt, nt + nq, nfq, tid_);
    for (uint32_t i = 0; i < nq; i++) {
        if (cnt_q[i] == nt || cnt_q[i] == 0) continue;
        const uint32_t s0 = (uint32_t)targets.size();
        for (uint32_t j = 0; j < nt; j++)
            if (!sw[(size_t)i * nt + j]) targets.push_back(j);
        ub.add(i, nf_q(i), kUnitTgtSide1, s0, (uint32_t)targets.size(), nft, tid_);
    }
    for (uint32_t j = 0; j < nt; j++) {
        if (cnt_t[j] == nq || cnt_t[j] == 0) continue;
        const uint32_t s0 = (uint32_t)targets.size();
        for (uint32_t i = 0; i < nq; i++)
            if (sw[(size_t)i * nt + j]) targets.push_back(i);
        ub.add(j, nf_t(j), kUnitRefSide1, s0, (uint32_t)targets.size(), nfq, tid_);
    }
}

// Unit budget for a job of `total` filter pairs on `slots` resident CTAs:
// the configured budget, lowered (to no less than 2^16) for small jobs so
// that every CTA gets about four units.
inline uint64_t effective_unit_budget(uint64_t configured, uint64_t total, uint64_t slots) {
    const uint64_t fair = total / std::max<uint64_t>(1, 4 * slots);
    return std::min(configured, std::max<uint64_t>(1ull << 16, fair));
}


}  // namespace sdbfg
