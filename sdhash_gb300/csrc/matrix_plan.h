// matrix_plan.h -- work-unit construction for the batched comparison
// engine (k_matrix), shared by the set comparison entry points and the
// serving loop.  Host code only.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

#include "compare_kernels.h"

namespace sdbfg {

// Accumulates the work units of one reference digest over a run of target
// list entries, cutting a new unit when the work budget or the per-unit
// target limit is reached, and row-splitting single pairs above the budget.
struct UnitBuilder {
    std::vector<MatUnit> units;
    std::vector<uint64_t> work;  // per unit, for the largest-first order
    std::vector<MatSplit> split;
    uint64_t slots = 0;
    uint64_t budget;
    uint64_t filter_pairs = 0;
    explicit UnitBuilder(uint64_t w) : budget(std::max<uint64_t>(w, 1)) {}

    // targets [t0, t1) of list `tl`, nf(e) = filters of list entry e
    template <class NF, class ID>
    void add(uint32_t ref, uint32_t nref, uint32_t flags, uint32_t t0, uint32_t t1, NF nf, ID id) {
        uint32_t start = t0;
        uint64_t acc = 0;
        auto flush = [&](uint32_t end) {
            if (end > start) {
                units.push_back(MatUnit{ref, 0, nref, start, end, flags, 0, 0});
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
                    units.push_back(MatUnit{ref, r, r1, e, e + 1, flags | kUnitSplit, si, 0});
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

// Unit budget for a job of `total` filter pairs on `slots` resident CTAs:
// the configured budget, lowered (to no less than 2^16) for small jobs so
// that every CTA gets about four units.
inline uint64_t effective_unit_budget(uint64_t configured, uint64_t total, uint64_t slots) {
    const uint64_t fair = total / std::max<uint64_t>(1, 4 * slots);
    return std::min(configured, std::max<uint64_t>(1ull << 16, fair));
}


}  // namespace sdbfg
