// tp_warpnbr.cuh — warp-cooperative neighbour iteration (sm_103a).
//
// One warp owns 32 consecutive slots (query particles).  Lanes are grouped by their (cy, cz) cell
// row; for each of the 3^(d-1) neighbour rows the group's candidate slots form ONE contiguous range
// (cells are linearised x fastest), which the warp streams through shared memory 32 records at a
// time.  Every lane tests every staged candidate with a cheap FP32 distance on cell-relative
// offsets and appends hits to its own queue in shared memory; when some lane's queue may overflow
// (and at the end) all lanes drain their queues in lock-step through `flush`, so the expensive
// pair physics runs with (almost) full lanes instead of diverging per candidate.
//
// Visiting order per lane: rows in (dz, dy) order, slots ascending inside a row -- the
// PointNeighbors order (neighbour cells in CartesianIndices order, ascending index in a cell),
// which the FP64 sums therefore keep.
//
// Test records: float4 {ox, oy, oz, cx} with o = x - floor(x / cs) * cs32 (cell-relative offset,
// cs32 = FP32 cell size) and cx the x cell index (as a float, exact).  Queue entries carry the
// slot (27 bits) and the row code (dy, dz) in the top 5 bits.
#pragma once

#include <climits>

#include "tp_internal.cuh"

namespace tp {

constexpr int kQCap = 64;          // queue entries per lane
constexpr int kSlotBits = 27;      // max 2^27 particles per set
constexpr int kSlotMask = (1 << kSlotBits) - 1;

struct WarpSmem {
    float4 cand[32];
    int q[kQCap][32];
};

__device__ __forceinline__ void row_shift(int code, int& dy, int& dz) {
    dy = (code % 3) - 1;
    dz = (code / 3) - 1;
}

// Drains every lane's queue: calls f(entry) for the lane's entries, lanes in lock-step.
template <class F>
__device__ __forceinline__ void drain(WarpSmem& sm, int n, F& f) {
    const int lane = threadIdx.x & 31;
    const int mx = __reduce_max_sync(0xffffffffu, n);
    for (int k = 0; k < mx; ++k) {
        if (k < n) f(sm.q[k][lane]);
    }
    __syncwarp();
}

// `active`: the lane has a query particle; `c`: its cell; `oa`: its test record.
template <int ND, class F>
__device__ __forceinline__ void warp_neighbors(const GridDesc& g, float cs, bool active,
                                               const int c[3], float4 oa,
                                               const int* __restrict__ start,
                                               const float4* __restrict__ test, float sr2f,
                                               WarpSmem& sm, F& f) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int cnt = 0;
    const int yz = active ? (c[1] + g.n[1] * c[2]) : -1;
    unsigned todo = __ballot_sync(FULL, active);
    while (todo) {
        const int leader = __ffs(todo) - 1;
        const int yz0 = __shfl_sync(FULL, yz, leader);
        const bool ing = active && (yz == yz0);
        const unsigned grp = __ballot_sync(FULL, ing);
        todo &= ~grp;
        const int cxmin = __reduce_min_sync(FULL, ing ? c[0] : INT_MAX);
        const int cxmax = __reduce_max_sync(FULL, ing ? c[0] : INT_MIN);
        const int cy = yz0 % g.n[1], cz = yz0 / g.n[1];
        const float cxa = (float)c[0];
        const int zlo = (ND == 3) ? -1 : 0, zhi = (ND == 3) ? 1 : 0;
        for (int dz = zlo; dz <= zhi; ++dz) {
            for (int dy = -1; dy <= 1; ++dy) {
                const int rb = g.n[0] * ((cy + dy) + g.n[1] * (cz + dz));
                const int lo = start[rb + cxmin - 1];
                const int hi = start[rb + cxmax + 2];
                if (lo >= hi) continue;
                int mlo = 0, mhi = 0;
                if (ing) {
                    mlo = start[rb + c[0] - 1];
                    mhi = start[rb + c[0] + 2];
                }
                const float sy = oa.y - (float)dy * cs;
                const float sz = oa.z - (float)dz * cs;
                const int code = ((dy + 1) + 3 * (dz + 1)) << kSlotBits;
                for (int base = lo; base < hi; base += 32) {
                    const int j = base + lane;
                    if (j < hi) sm.cand[lane] = test[j];
                    __syncwarp();
                    const int nc = min(32, hi - base);
                    for (int k = 0; k < nc; ++k) {
                        const float4 cb = sm.cand[k];
                        const int jj = base + k;
                        const float pdx = fmaf(cxa - cb.w, cs, oa.x) - cb.x;
                        const float pdy = sy - cb.y;
                        float d2 = pdx * pdx + pdy * pdy;
                        if (ND == 3) {
                            const float pdz = sz - cb.z;
                            d2 = fmaf(pdz, pdz, d2);
                        }
                        if (jj >= mlo && jj < mhi && d2 <= sr2f) {
                            sm.q[cnt][lane] = jj | code;
                            ++cnt;
                        }
                    }
                    __syncwarp();
                    if (__any_sync(FULL, cnt > kQCap - 32)) {
                        drain(sm, cnt, f);
                        cnt = 0;
                    }
                }
            }
        }
    }
    if (__any_sync(FULL, cnt > 0)) drain(sm, cnt, f);
}

// Test record of a point (FP64 coordinates) for a grid with FP64 cell size cs and FP32 cs32.
template <int ND>
__device__ __forceinline__ float4 test_record(const double* x, const GridDesc& g, double cs32) {
    float o[3] = {0.0f, 0.0f, 0.0f};
    float cx = 0.0f;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const double fl = floor(__ddiv_rn(x[d], g.cs));
        o[d] = (float)__dsub_rn(x[d], __dmul_rn(fl, cs32));
        if (d == 0) cx = (float)(fl - (double)g.cmin[0]);
    }
    return make_float4(o[0], o[1], o[2], cx);
}

}  // namespace tp
