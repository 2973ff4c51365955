// tp_lists.cuh — per-step neighbour lists (Verlet lists with a skin) on sm_103a.
//
// A list holds, for every query slot, the candidates within r_list = 2h (1 + skin) at the time
// of the last cell-list rebuild.  Pairs are still decided exactly at use time
// (|x_a - x_b|^2 <= (2h)^2 with the current positions), so the neighbour set is unchanged as long
// as no particle has moved more than skin * h since the rebuild; the displacement check below
// reopens the rebuild gate before that can happen (see tp_nhs.cuh for the gate).
//
// Layout: entry k of slot s at list[k * stride + s] (stride = number of query slots), so the 32
// lanes of a warp read one 128-byte line per k.  An entry is the candidate slot (27 bits) and
// the candidate's cell offset code (dx+1) + 3(dy+1) + 9(dz+1) relative to the query's cell at
// build time (top 5 bits), which the FP32 form needs to form cell-relative differences.
// Entries are in PointNeighbors visiting order (rows in (dz, dy) order, ascending slots).
#pragma once

#include "tp_nhs.cuh"
#include "tp_warpnbr.cuh"

namespace tp {

#define TP_ERRBIT_CAPACITY 4

__device__ __forceinline__ void decode_cell_offset(unsigned e, int& dx, int& dy, int& dz) {
    const int code = (int)(e >> kSlotBits);
    dx = code % 3 - 1;
    dy = (code / 3) % 3 - 1;
    dz = code / 9 - 1;
}

// o_a - o_b + (c_a - c_b) * cs from a list entry (same arithmetic as the list filter).
template <int ND>
__device__ __forceinline__ float pair_diff(float4 ta, float cs, unsigned e, float4 cb, float& pdx,
                                           float& pdy, float& pdz) {
    int dx, dy, dz;
    decode_cell_offset(e, dx, dy, dz);
    pdx = fmaf(-(float)dx, cs, ta.x) - cb.x;
    pdy = fmaf(-(float)dy, cs, ta.y) - cb.y;
    float d2 = fmaf(pdy, pdy, pdx * pdx);
    pdz = 0.0f;
    if (ND == 3) {
        pdz = fmaf(-(float)dz, cs, ta.z) - cb.z;
        d2 = fmaf(pdz, pdz, d2);
    }
    return d2;
}

// Largest displacement since the last rebuild -> gate[1] (float bits, atomicMax on unsigned).
template <int ND>
__global__ void __launch_bounds__(256) k_displacement(const double* __restrict__ u,
                                                      const double* __restrict__ xb, int n,
                                                      unsigned* __restrict__ gate) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    float d = 0.0f;
    if (s < n) {
        double d2 = 0.0;
#pragma unroll
        for (int k = 0; k < ND; ++k) {
            const double e = u[(size_t)s * ND + k] - xb[(size_t)s * ND + k];
            d2 += e * e;
        }
        d = (float)sqrt(d2);
        if (!(d == d)) d = 3.0e38f;  // NaN positions force a rebuild (and are reported there)
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, off));
    if ((threadIdx.x & 31) == 0 && d > 0.0f) atomicMax(&gate[1], __float_as_uint(d));
}

// Same staging loop as warp_neighbors, but every hit goes straight into the lane's list column.
template <int ND>
__device__ __forceinline__ int warp_collect(const GridDesc& g, float cs, bool active,
                                            const int c[3], float4 oa,
                                            const int* __restrict__ start,
                                            const float4* __restrict__ test, float r2f,
                                            float4* cand, unsigned* __restrict__ list,
                                            int stride, int cap, int s) {
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
                const float sy = fmaf(-(float)dy, cs, oa.y);
                const float sz = fmaf(-(float)dz, cs, oa.z);
                const unsigned rowcode = (unsigned)(3 * (dy + 1) + 9 * (dz + 1));
                for (int base = lo; base < hi; base += 32) {
                    const int j = base + lane;
                    if (j < hi) cand[lane] = test[j];
                    __syncwarp();
                    const int nc = min(32, hi - base);
                    for (int k = 0; k < nc; ++k) {
                        const float4 cb = cand[k];
                        const int jj = base + k;
                        const float pdx = fmaf(cxa - cb.w, cs, oa.x) - cb.x;
                        const float pdy = sy - cb.y;
                        float d2 = fmaf(pdy, pdy, pdx * pdx);
                        if (ND == 3) {
                            const float pdz = sz - cb.z;
                            d2 = fmaf(pdz, pdz, d2);
                        }
                        if (jj >= mlo && jj < mhi && d2 <= r2f) {
                            const unsigned code = rowcode + (unsigned)((int)(cb.w - cxa) + 1);
                            if (cnt < cap) list[(size_t)cnt * stride + s] = (unsigned)jj | (code << kSlotBits);
                            ++cnt;
                        }
                    }
                    __syncwarp();
                }
            }
        }
    }
    return cnt;
}

// Fluid slots: fluid-fluid and fluid-wall lists.
template <int ND>
__global__ void __launch_bounds__(128) k_build_fluid_lists(
    GridDesc g, float cs, float r2f, int nf, const float4* __restrict__ ftest,
    const int* __restrict__ fskey, const int* __restrict__ fstart,
    const float4* __restrict__ wtest, const int* __restrict__ wstart, unsigned* __restrict__ ff,
    int* __restrict__ ffc, int cap_ff, unsigned* __restrict__ fw, int* __restrict__ fwc,
    int cap_fw, int* __restrict__ err, const unsigned* __restrict__ gate) {
    if (!gate_open(gate)) return;
    __shared__ float4 cand_all[4][32];
    float4* cand = cand_all[threadIdx.x >> 5];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s < nf;
    const int si = active ? s : 0;
    const float4 ta = ftest[si];
    int c[3];
    key_to_coords(fskey[si], g, c);
    const int n1 = warp_collect<ND>(g, cs, active, c, ta, fstart, ftest, r2f, cand, ff, nf,
                                    cap_ff, s);
    const int n2 = warp_collect<ND>(g, cs, active, c, ta, wstart, wtest, r2f, cand, fw, nf,
                                    cap_fw, s);
    if (!active) return;
    ffc[s] = min(n1, cap_ff);
    fwc[s] = min(n2, cap_fw);
    if (n1 > cap_ff || n2 > cap_fw) atomicOr(err, TP_ERRBIT_CAPACITY);
}

// Wall slots: wall-fluid lists (the Adami gather).
template <int ND>
__global__ void __launch_bounds__(128) k_build_wall_lists(
    GridDesc g, float cs, float r2f, int nw, const float4* __restrict__ wtest,
    const int* __restrict__ wskey, const float4* __restrict__ ftest,
    const int* __restrict__ fstart, unsigned* __restrict__ wf, int* __restrict__ wfc, int cap_wf,
    int* __restrict__ err, const unsigned* __restrict__ gate) {
    if (!gate_open(gate)) return;
    __shared__ float4 cand_all[4][32];
    float4* cand = cand_all[threadIdx.x >> 5];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s < nw;
    const int si = active ? s : 0;
    const float4 ta = wtest[si];
    int c[3];
    key_to_coords(wskey[si], g, c);
    const int n1 = warp_collect<ND>(g, cs, active, c, ta, fstart, ftest, r2f, cand, wf, nw,
                                    cap_wf, s);
    if (!active) return;
    wfc[s] = min(n1, cap_wf);
    if (n1 > cap_wf) atomicOr(err, TP_ERRBIT_CAPACITY);
}

// Largest cell occupancy of a freshly counted histogram (list capacity sizing).
static __global__ void k_max_count(const int* __restrict__ count, int n, int* __restrict__ out) {
    int m = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        m = max(m, count[i]);
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(out, m);
}

// Test record of point x relative to the cell `key` (offsets against the FP32 cell size).
template <int ND>
__device__ __forceinline__ float4 test_record_in(const double* x, const GridDesc& g, double cs32,
                                                 int key) {
    int c[3];
    key_to_coords(key, g, c);
    float o[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int d = 0; d < ND; ++d)
        o[d] = (float)__dsub_rn(x[d], __dmul_rn((double)(g.cmin[d] + c[d]), cs32));
    return make_float4(o[0], o[1], o[2], (float)c[0]);
}

}  // namespace tp
