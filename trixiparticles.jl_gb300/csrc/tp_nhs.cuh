// tp_nhs.cuh — cell-list neighbour search as a counting sort by cell (sm_103a).
//
// Replaces PointNeighbors' GridNeighborhoodSearch update for a FullGridCellList (called from
// update_nhs!, src/general/neighborhood_search.jl:479-519, 804-808).  One rebuild is four
// passes over the particles:
//   1. keys     — cell key per particle + cell histogram with warp-aggregated atomics
//                 (__match_any_sync groups lanes with the same key; one atomic per group);
//   2. scan     — exclusive prefix scan of the histogram -> first slot of every cell
//                 (three-kernel reduce / scan-partials / scan-and-write scan);
//   3. scatter  — warp-aggregated atomic claim of slots inside each cell;
//   4. rank     — deterministic fix-up: a particle's final slot inside its cell is its rank by
//                 source index among the cell's particles, so the sorted order is the stable
//                 order (cell, index) whatever order the atomics ran in; the same pass packs
//                 the particle's record into its slot (SoA reorder).
// The scan also re-zeroes the histogram, so no memset is needed between rebuilds.
//
// Gate: inside the integrator the cell list is rebuilt only when some particle has moved more
// than half the neighbour-list skin since the last rebuild (or a rebuild is forced).  The
// decision is taken on the device: gate[0] = force flag, gate[1] = largest squared displacement
// since the last rebuild (non-negative float bits, so unsigned order = float order), gate[2] =
// the squared half skin (skin * h)^2, lowered by 1e-5 relative so that FP32 rounding of the
// displacement never lets a particle past the margin unseen (float bits).  A null gate means
// "always rebuild".  When the gate is closed the kernels return at once and the rank pass packs
// every slot in place.  gate[4] counts the rebuilds the gate has let through since the handle was
// created (the key pass bumps it once per open gate).
#pragma once

#include "tp_internal.cuh"

namespace tp {

__device__ __forceinline__ bool gate_open(const unsigned* gate) {
    return gate == nullptr || gate[0] != 0u || gate[1] > gate[2];
}

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// LEX: key with z fastest, i.e. lexicographic order of (cx, cy, cz) -- the order of Julia's
// sortperm over SVector cell coordinates (SortingCallback); default: x fastest (the cell list).
template <int ND, bool LEX = false>
__global__ void __launch_bounds__(256) k_cell_keys(const double* __restrict__ u, int n,
                                                   GridDesc g, int* __restrict__ key,
                                                   int* __restrict__ count, int* __restrict__ err,
                                                   const unsigned* __restrict__ gate = nullptr) {
    if (!gate_open(gate)) return;
    // gate[4] counts the rebuilds the gate let through (diagnostics, tp_rebuild_count)
    if (gate && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(const_cast<unsigned*>(gate) + 4, 1u);
    // any grid: the blocks stride over the particles (block-uniform trip count)
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        const bool valid = i < n;
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        double x[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < ND; ++d) x[d] = u[(size_t)i * ND + d];
        int c[3];
        const int e = cell_coords<ND>(x, g, c);
        if (e) atomicOr(err, e);
        const int k = LEX ? c[2] + g.n[2] * (c[1] + g.n[1] * c[0]) : cell_key(c, g);
        key[i] = k;
        const unsigned peers = __match_any_sync(vmask, k);
        if (lane_id() == __ffs(peers) - 1) atomicAdd(&count[k], __popc(peers));
    }
}

// Block-wide exclusive scan of kScanItems values per thread; returns the block total.
__device__ __forceinline__ int block_exclusive_scan(int (&v)[kScanItems], int* warp_sums) {
    int local = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        int t = v[j];
        v[j] = local;
        local += t;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = local;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int ws = (lane < (kScanThreads >> 5)) ? warp_sums[lane] : 0;
        int wincl = ws;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, wincl, off);
            if (lane >= off) wincl += y;
        }
        warp_sums[lane] = wincl - ws;  // exclusive
        if (lane == 31) warp_sums[32] = wincl;
    }
    __syncthreads();
    const int base = warp_sums[warp] + (incl - local);
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) v[j] += base;
    const int total = warp_sums[32];
    __syncthreads();
    return total;
}

// Per-tile sums of the histogram.  Any grid: the blocks walk the tiles (tile = blockIdx.x,
// + gridDim.x, ...), so that a closed gate costs one short launch over a large grid of cells.
static __global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int* __restrict__ count, int n,
                                                             int* __restrict__ partial,
                                                             const unsigned* __restrict__ gate = nullptr) {
    if (!gate_open(gate)) return;
    __shared__ int sm[33];
    const int nb = (n + kScanTile - 1) / kScanTile;
    for (int tile = blockIdx.x; tile < nb; tile += gridDim.x) {
        const int base = tile * kScanTile;
        int s = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            int idx = base + j * kScanThreads + threadIdx.x;
            if (idx < n) s += count[idx];
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            int t = (threadIdx.x < (kScanThreads >> 5)) ? sm[threadIdx.x] : 0;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
            if (threadIdx.x == 0) partial[tile] = t;
        }
        __syncthreads();  // sm is reused by the next tile
    }
}

// Single block: exclusive scan of the per-tile partial sums, in chunks of kScanTile.
static __global__ void __launch_bounds__(kScanThreads) k_scan_partials(int* __restrict__ partial, int nb,
                                                               const unsigned* __restrict__ gate = nullptr) {
    if (!gate_open(gate)) return;
    __shared__ int ws[33];
    int carry = 0;
    for (int base = 0; base < nb; base += kScanTile) {
        int v[kScanItems];
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            int idx = base + threadIdx.x * kScanItems + j;
            v[j] = (idx < nb) ? partial[idx] : 0;
        }
        int total = block_exclusive_scan(v, ws);
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            int idx = base + threadIdx.x * kScanItems + j;
            if (idx < nb) partial[idx] = v[j] + carry;
        }
        carry += total;
        __syncthreads();
    }
}

// start[c] = exclusive prefix of count; cursor[c] = start[c]; count[c] = 0; start[n] = total.
// Any grid, as k_scan_reduce.
static __global__ void __launch_bounds__(kScanThreads) k_scan_final(int* __restrict__ count, int n,
                                                            const int* __restrict__ partial,
                                                            int* __restrict__ start,
                                                            int* __restrict__ cursor,
                                                            const unsigned* __restrict__ gate = nullptr) {
    if (!gate_open(gate)) return;
    __shared__ int ws[33];
    const int nb = (n + kScanTile - 1) / kScanTile;
    for (int tile = blockIdx.x; tile < nb; tile += gridDim.x) {
        const int base = tile * kScanTile + threadIdx.x * kScanItems;
        int v[kScanItems];
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) v[j] = (base + j < n) ? count[base + j] : 0;
        const int total = block_exclusive_scan(v, ws);
        const int off = partial[tile];
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            int idx = base + j;
            if (idx < n) {
                start[idx] = v[j] + off;
                if (cursor) cursor[idx] = v[j] + off;
                count[idx] = 0;
            }
        }
        if (tile == nb - 1 && threadIdx.x == 0) start[n] = off + total;
    }
}

static __global__ void __launch_bounds__(256) k_scatter(const int* __restrict__ key, int n,
                                                 int* __restrict__ cursor, int* __restrict__ tmp,
                                                 const unsigned* __restrict__ gate = nullptr) {
    if (!gate_open(gate)) return;
    for (int b0 = blockIdx.x * blockDim.x; b0 < n; b0 += gridDim.x * blockDim.x) {
        const int i = b0 + threadIdx.x;
        const bool valid = i < n;
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        const int k = key[i];
        const unsigned peers = __match_any_sync(vmask, k);
        const int leader = __ffs(peers) - 1;
        int base = 0;
        if (lane_id() == leader) base = atomicAdd(&cursor[k], __popc(peers));
        base = __shfl_sync(peers, base, leader);
        tmp[base + __popc(peers & lanemask_lt())] = i;
    }
}

// Final slot = cell start + rank of the source index among the cell's particles.  The packer
// functor copies source particle i into slot dst of cell `key` (records, masses, state).  With
// a closed gate every slot is packed in place: pack(s, s, skey[s]).
template <class Packer>
__global__ void __launch_bounds__(256) k_rank_pack(const int* __restrict__ tmp,
                                                   const int* __restrict__ key,
                                                   const int* __restrict__ start, int n,
                                                   int* __restrict__ perm, int* __restrict__ skey,
                                                   Packer pack,
                                                   const unsigned* __restrict__ gate = nullptr) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    if (!gate_open(gate)) {
        pack(s, s, skey[s], false);
        return;
    }
    const int i = tmp[s];
    const int k = key[i];
    const int lo = start[k], hi = start[k + 1];
    int r = 0;
    for (int j = lo; j < hi; ++j) r += (tmp[j] < i);
    const int dst = lo + r;
    perm[dst] = i;
    skey[dst] = k;
    pack(i, dst, k, true);
}

// Rank pass without packing (wall setup and diagnostics).
struct NoPack {
    __device__ void operator()(int, int, int, bool) const {}
};

}  // namespace tp
