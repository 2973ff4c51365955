// tp_lists.cuh — per-step neighbour lists (Verlet lists with a skin) on sm_103a.
//
// A list holds, for every query slot, the candidates within r_list = 2h (1 + skin) at the time
// of the last cell-list rebuild.  Pairs are still decided exactly at use time
// (|x_a - x_b|^2 <= (2h)^2 with the current positions), so the neighbour set is unchanged as long
// as no particle has moved more than skin * h since the rebuild; the displacement check below
// reopens the rebuild gate before that can happen (see tp_nhs.cuh for the gate).
//
// Layout: a slot's entries come in chunks of eight, chunk q of slot s at entries
// [(q * stride + s) * 8, + 8) (stride = number of query slots): a builder lane writes one whole
// 32-byte sector per chunk (scattered 4-byte appends into a slot-interleaved layout cost the
// builder 3.4x its time in partial-sector writes), and a reader lane fetches four consecutive
// entries with one 16-byte load (a warp's quad read covers half of 32 adjacent sectors, whose
// other halves the next quad reads).  An entry is the candidate slot (25 bits) and the
// candidate's cell offset code (dx+2) + 5(dy+2) + 25(dz+2) relative to the query's cell at
// build time (top 7 bits), which the FP32 form needs to form cell-relative differences.
//
// Cells are 2h wide (the reference's grid) and the list radius 2h (1 + skin) is larger, so a
// query within 2h skin of a cell face can have candidates two cells away along that axis: the
// search covers +-1 cells always and +-2 along an axis whenever the query's offset lies within
// r_list - cs of the corresponding face.  Entries are in CartesianIndices order of the searched
// cells (rows in (dz, dy) order, ascending slots within a row), so the pairs within 2h -- all in
// the +-1 cells -- keep the PointNeighbors visiting order.
#pragma once

#include <climits>

#include "tp_nhs.cuh"

namespace tp {

#define TP_ERRBIT_CAPACITY 4

constexpr int kSlotBits = 25;  // slot field of a list entry: at most 2^25 particles per set
constexpr int kListChunk = 8;  // entries per chunk; list capacities are multiples of it

__host__ __device__ __forceinline__ size_t list_at(int k, int stride, int s) {
    return ((size_t)(k >> 3) * (size_t)stride + (size_t)s) * kListChunk + (size_t)(k & 7);
}

// Entries k .. k+3 of slot s (k a multiple of 4).
__device__ __forceinline__ uint4 list_quad(const unsigned* __restrict__ list, int k, int stride,
                                           int s) {
    return *reinterpret_cast<const uint4*>(list + list_at(k, stride, s));
}

// The same for a pass that reads each list entry once: the quad is not allocated in L1, which
// keeps L1 for the neighbour records the pass gathers (ld.global.nc with L1::no_allocate).
__device__ __forceinline__ uint4 list_quad_stream(const unsigned* __restrict__ list, int k,
                                                  int stride, int s) {
    uint4 q;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(q.x), "=r"(q.y), "=r"(q.z), "=r"(q.w)
        : "l"(list + list_at(k, stride, s)));
    return q;
}

// The same for a list written earlier in the same kernel by the reading thread (the exact pair
// lists of the fused FP64 pass): plain loads, never the read-only data path.
__device__ __forceinline__ unsigned list_next_rw(const unsigned* list, int k, int stride, int s,
                                                 uint4& q) {
    if ((k & 3) == 0) q = *reinterpret_cast<const uint4*>(list + list_at(k, stride, s));
    const int r = k & 3;
    return r == 0 ? q.x : r == 1 ? q.y : r == 2 ? q.z : q.w;
}

constexpr unsigned kSlotMask = (1u << kSlotBits) - 1u;

// Cell offsets of the 125 entry codes times the FP32 cell size, {dx cs, dy cs, dz cs, 0} at
// code (dx+2) + 5 (dy+2) + 25 (dz+2), staged in shared memory by every kernel that reads lists:
// one 16-byte shared load per candidate instead of an integer-division decode.  dx cs is exact
// in FP32 for |dx| <= 2, so (o_a - dx cs) rounds exactly like fmaf(-dx, cs, o_a).
constexpr int kOffsetCodes = 125;

// Fills the block's table and synchronises the block: call before any thread returns.
__device__ __forceinline__ void fill_offset_table(float4* tab, float cs) {
    for (int i = threadIdx.x; i < kOffsetCodes; i += blockDim.x)
        tab[i] = make_float4((float)(i % 5 - 2) * cs, (float)((i / 5) % 5 - 2) * cs,
                             (float)(i / 25 - 2) * cs, 0.0f);
    __syncthreads();
}

// Reach of the cell search of a query at offset o in its cell along one axis: 2 cells towards a
// face closer than m = r_list - cs, else 1.
__device__ __forceinline__ int reach_lo(float o, float m) { return o <= m ? 2 : 1; }
__device__ __forceinline__ int reach_hi(float o, float cs, float m) { return o >= cs - m ? 2 : 1; }

// o_a - o_b + (c_a - c_b) * cs from a list entry and the block's offset table (same arithmetic
// as the list filter).
template <int ND>
__device__ __forceinline__ float pair_diff(float4 ta, const float4* tab, unsigned e, float4 cb,
                                           float& pdx, float& pdy, float& pdz) {
    const float4 o = tab[e >> kSlotBits];
    pdx = (ta.x - o.x) - cb.x;
    pdy = (ta.y - o.y) - cb.y;
    float d2 = fmaf(pdy, pdy, pdx * pdx);
    pdz = 0.0f;
    if (ND == 3) {
        pdz = (ta.z - o.z) - cb.z;
        d2 = fmaf(pdz, pdz, d2);
    }
    return d2;
}

// The cell offset of a list entry as FP32 multiples of the cell size, decoded arithmetically
// from the code (dx+2) + 5 (dy+2) + 25 (dz+2) (exact for the 125 codes: the digits come from
// floor((c + 1/2) / 25) and floor((r + 1/2) / 5) in FP32), so that pair differences can be formed
// without the shared offset table: (o_a - d cs) is fmaf(-d, cs, o_a), the table's rounding.
__device__ __forceinline__ void entry_cell_offset(unsigned e, float& fx, float& fy, float& fz) {
    const float c = (float)(e >> kSlotBits);
    fz = floorf(fmaf(c, 0.04f, 0.02f));
    const float r = fmaf(-25.0f, fz, c);
    fy = floorf(fmaf(r, 0.2f, 0.1f));
    fx = fmaf(-5.0f, fy, r) - 2.0f;
    fy -= 2.0f;
    fz -= 2.0f;
}

template <int ND>
__device__ __forceinline__ float pair_diff_decoded(float4 ta, float cs, unsigned e, float4 cb,
                                                   float& pdx, float& pdy, float& pdz) {
    float fx, fy, fz;
    entry_cell_offset(e, fx, fy, fz);
    pdx = fmaf(-fx, cs, ta.x) - cb.x;
    pdy = fmaf(-fy, cs, ta.y) - cb.y;
    float d2 = fmaf(pdy, pdy, pdx * pdx);
    pdz = 0.0f;
    if (ND == 3) {
        pdz = fmaf(-fz, cs, ta.z) - cb.z;
        d2 = fmaf(pdz, pdz, d2);
    }
    return d2;
}

// Squared displacement of one particle, the same arithmetic as k_displacement: FP64 differences
// rounded to FP32, FP32 sum of squares.
template <int ND>
__device__ __forceinline__ float displacement2(const double* x, const double* __restrict__ xb) {
    float d2 = 0.0f;
#pragma unroll
    for (int k = 0; k < ND; ++k) {
        const float e = (float)(x[k] - xb[k]);
        d2 = fmaf(e, e, d2);
    }
    return (d2 == d2) ? d2 : 3.0e38f;  // NaN positions force a rebuild (and are reported there)
}

// The integrator's pair stage already holds every particle's next position: it folds the
// displacement check of the next stage into its update, each converged group of lanes taking
// the maximum of its squared displacements into `word` (float bits, atomicMax on unsigned);
// lanes that returned early take no part.
__device__ __forceinline__ void gate_max_displacement(unsigned* word, float d2) {
    const unsigned m = __activemask();
    const unsigned mx = __reduce_max_sync(m, __float_as_uint(d2));
    if ((int)(threadIdx.x & 31) == __ffs(m) - 1 && mx > 0u) atomicMax(word, mx);
}

// Largest squared displacement since the last rebuild -> gate[1] (float bits, atomicMax on
// unsigned), compared with the squared threshold in gate[2].  Only the differences are FP64 (the
// positions are); squares and sum are FP32 and there is no square root: the pass was bound by
// the FP64 pipe (sqrt of the FP64 distance).  The threshold is lowered by 1e-5 relative to cover
// the FP32 rounding, so a rebuild never comes later than the exact test would have it.
// `perm` (optional): slot -> index into u (caller-ordered positions of the kick! path).
template <int ND>
__global__ void __launch_bounds__(256) k_displacement(const double* __restrict__ u,
                                                      const double* __restrict__ xb, int n,
                                                      unsigned* __restrict__ gate,
                                                      const int* __restrict__ perm = nullptr) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.0f;
    if (s < n) {
        const int i = perm ? perm[s] : s;
        d2 = displacement2<ND>(u + (size_t)i * ND, xb + (size_t)s * ND);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) d2 = fmaxf(d2, __shfl_xor_sync(0xffffffffu, d2, off));
    if ((threadIdx.x & 31) == 0 && d2 > 0.0f) atomicMax(&gate[1], __float_as_uint(d2));
}

// The packed FP32 arithmetic of sm_100+: one FFMA2, FADD2 or FMUL2 computes both halves of a
// float2, each rounded as the scalar operation.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.0f), a); }

// Staging buffer of one warp of the candidate search: up to 32 compacted records as {slot, x
// cell} and separate coordinate arrays, so that two consecutive entries load as one int4 / float2
// (two spare entries keep those loads in bounds).
struct __align__(16) SearchStage {
    int2 jc[34];
    float x[34], y[34], z[34];
};

// Widest x extent (in cells beyond the first) of a lane group of the candidate search.
constexpr int kGroupSpan = 2;

// Warp-cooperative candidate search: lanes are grouped by their (cy, cz) row; for each searched
// row the group's candidates form one contiguous slot range (cells are linearised x fastest),
// which the warp streams through shared memory 32 test records at a time, and every lane tests
// the staged records against its own cell range and radius and appends hits to its list column.
// m = r_list - cs (plus a rounding margin) decides where the search reaches two cells.
//
// Because a cell's particles fill it, some lane of a group is nearly always close to each face,
// so the union of the lanes' ranges is about 5 x 5 rows of 5 cells.  The group's lanes are
// therefore bounded by a box (relative to the group's first cell), rows farther than r_list from
// the box are skipped, and each staged record is first tested against the box inflated by
// r_list (by the lane that staged it); only records that pass are tested by every lane.  The box
// tests are conservative (inflated radius and margins), so the lists -- entries and order -- are
// the ones the plain union search produces.
template <int ND>
__device__ __forceinline__ int warp_collect(const GridDesc& g, float cs, float m, bool active,
                                            const int c[3], float4 oa,
                                            const int* __restrict__ start,
                                            const int* __restrict__ skey,
                                            const float4* __restrict__ test, int tstride,
                                            float r2f,
                                            SearchStage* st, unsigned* lbuf,
                                            unsigned* __restrict__ list, int stride, int cap,
                                            int s) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int cnt = 0;
    // a lane's entries are collected in its column of the block's buffer (entry r of the open
    // chunk at lbuf[r * blockDim.x]) and written out a whole chunk at a time
    const int bs = blockDim.x;
    auto flush = [&](int q) {
        uint4* dst = reinterpret_cast<uint4*>(list + list_at(q * kListChunk, stride, s));
        dst[0] = make_uint4(lbuf[0], lbuf[bs], lbuf[2 * bs], lbuf[3 * bs]);
        dst[1] = make_uint4(lbuf[4 * bs], lbuf[5 * bs], lbuf[6 * bs], lbuf[7 * bs]);
    };
    const int xl = reach_lo(oa.x, m), xh = reach_hi(oa.x, cs, m);
    const int yl = reach_lo(oa.y, m), yh = reach_hi(oa.y, cs, m);
    const int zl = (ND == 3) ? reach_lo(oa.z, m) : 0, zh = (ND == 3) ? reach_hi(oa.z, cs, m) : 0;
    const int yz = active ? (c[1] + g.n[1] * c[2]) : -1;
    const float margin = 1e-3f * cs;
    const float rbox = sqrtf(r2f) * 1.0001f + margin;
    const float r2box = rbox * rbox;
    unsigned todo = __ballot_sync(FULL, active);
    while (todo) {
        // a group: the lowest pending lane and the pending lanes of its row at most kGroupSpan
        // cells further along x (slot order puts them after it), so that a warp whose slots sit
        // at both ends of a row (the two side walls of a tank) does not search the whole row
        const int leader = __ffs(todo) - 1;
        const int yz0 = __shfl_sync(FULL, yz, leader);
        const int cx0 = __shfl_sync(FULL, c[0], leader);
        const bool ing = active && ((todo >> lane) & 1u) && (yz == yz0) && (c[0] - cx0 <= kGroupSpan);
        const unsigned grp = __ballot_sync(FULL, ing);
        todo &= ~grp;
        const int cy = yz0 % g.n[1], cz = yz0 / g.n[1];
        // x of the lane relative to the group's first cell cx0 (staged records carry the same)
        const float xlane = fmaf((float)(c[0] - cx0), cs, oa.x);
        // box of the group's lanes relative to cell (cx0, cy, cz); the group's cells are
        // cx >= cx0 (slot order), offsets are clamped at 0 so that float bits order as ints
        const float ax = fmaxf(xlane, 0.0f);
        const float ay = fmaxf(oa.y, 0.0f), az = fmaxf(oa.z, 0.0f);
        // min / max over the group's lanes of non-negative floats, as ints
        auto gmin = [&](float x) {
            return __int_as_float(__reduce_min_sync(FULL, ing ? __float_as_int(x) : INT_MAX));
        };
        auto gmax = [&](float x) {
            return __int_as_float(__reduce_max_sync(FULL, ing ? __float_as_int(x) : 0));
        };
        const float bx0 = gmin(ax) - margin, bx1 = gmax(ax) + margin;
        const float by0 = gmin(ay) - margin, by1 = gmax(ay) + margin;
        float bz0 = 0.0f, bz1 = 0.0f;
        if (ND == 3) {
            bz0 = gmin(az) - margin;
            bz1 = gmax(az) + margin;
        }
        // distance of a row's slab [d cs, (d + 1) cs] from the box [b0, b1] along one axis
        auto slab = [&](int d, float b0, float b1) {
            return fmaxf(fmaxf((float)d * cs - b1, b0 - (float)(d + 1) * cs), 0.0f);
        };
        const int zr = (ND == 3) ? 2 : 0;
        for (int dz = -zr; dz <= zr; ++dz) {
            if (cz + dz < 0 || cz + dz >= g.n[2]) continue;
            const float ez = (ND == 3) ? slab(dz, bz0, bz1) : 0.0f;
            for (int dy = -2; dy <= 2; ++dy) {
                if (cy + dy < 0 || cy + dy >= g.n[1]) continue;
                const float ey = slab(dy, by0, by1);
                if (fmaf(ey, ey, ez * ez) > r2box) continue;  // the whole row is out of reach
                const bool need = ing && dy >= -yl && dy <= yh && dz >= -zl && dz <= zh;
                if (!__ballot_sync(FULL, need)) continue;
                const int xa = need ? max(c[0] - xl, 0) : INT_MAX;
                const int xb = need ? min(c[0] + xh, g.n[0] - 1) : INT_MIN;
                const int gxa = __reduce_min_sync(FULL, xa);
                const int gxb = __reduce_max_sync(FULL, xb);
                const int rb = g.n[0] * ((cy + dy) + g.n[1] * (cz + dz));
                const int lo = start[rb + gxa];
                const int hi = start[rb + gxb + 1];
                if (lo >= hi) continue;
                int mlo = 0, mhi = 0;
                if (need) {
                    mlo = start[rb + xa];
                    mhi = start[rb + xb + 1];
                }
                const float sy = fmaf(-(float)dy, cs, oa.y);
                const float sz = fmaf(-(float)dz, cs, oa.z);
                const float2 xl2 = f2(xlane), sy2 = f2(sy), sz2 = f2(sz);
                const float ryz = fmaf(ey, ey, ez * ez);
                const unsigned rowcode = 5u * (unsigned)(dy + 2) + 25u * (unsigned)(dz + 2);
                // the next chunk's records are loaded while the current one is tested
                float4 nxt = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                int nkey = 0;
                if (lo + lane < hi) {
                    nxt = test[(size_t)(lo + lane) * tstride];
                    nkey = skey[lo + lane];
                }
                for (int base = lo; base < hi; base += 32) {
                    const int j = base + lane;
                    bool rel = false;
                    float4 cb = nxt;
                    const int key = nkey;
                    int cxb = 0;
                    if (j + 32 < hi) {
                        nxt = test[(size_t)(j + 32) * tstride];
                        nkey = skey[j + 32];
                    }
                    if (j < hi) {
                        // offsets from the test record, the x cell from the sorted cell key
                        // (the record's fourth slot carries per-stage data in the FP32 form);
                        // staged as {x relative to cx0, oy, oz} and {slot, x cell} so that the
                        // lanes' tests below need no conversions
                        cxb = key - rb;
                        const float X = fmaf((float)(cxb - cx0), cs, cb.x);
                        cb.x = X;
                        // box distance of the staged record (its row distance is ey, ez at least)
                        const float Y = fmaf((float)dy, cs, cb.y);
                        const float ex = fmaxf(fmaxf(bx0 - X, X - bx1), 0.0f);
                        const float eyc = fmaxf(fmaxf(by0 - Y, Y - by1), 0.0f);
                        float d2b = fmaf(ex, ex, eyc * eyc);
                        if (ND == 3) {
                            const float Z = fmaf((float)dz, cs, cb.z);
                            const float ezc = fmaxf(fmaxf(bz0 - Z, Z - bz1), 0.0f);
                            d2b = fmaf(ezc, ezc, d2b);
                        }
                        rel = fmaxf(d2b, ryz) <= r2box;
                    }
                    // the records that pass are compacted in staging order (ballot prefix), so the
                    // test loop below reads them at consecutive shared addresses
                    const unsigned hits = __ballot_sync(FULL, rel);
                    if (rel) {
                        const int pos = __popc(hits & ((1u << lane) - 1u));
                        st->jc[pos] = make_int2(j, cxb);
                        st->x[pos] = cb.x;
                        st->y[pos] = cb.y;
                        st->z[pos] = cb.z;
                    }
                    __syncwarp();
                    // every lane tests the staged records, two per packed instruction (the scalar
                    // test's arithmetic), and appends its hits in staging order
                    const int nrel = __popc(hits);
                    auto append = [&](int jj, int cxj) {
                        const unsigned code = rowcode + (unsigned)(cxj - c[0] + 2);
                        if (cnt < cap) {
                            lbuf[(cnt & 7) * bs] = (unsigned)jj | (code << kSlotBits);
                            if ((cnt & 7) == 7) flush(cnt >> 3);
                        }
                        ++cnt;
                    };
                    for (int i = 0; i < nrel; i += 2) {
                        const float2 pdx = sub2(xl2, *reinterpret_cast<const float2*>(&st->x[i]));
                        const float2 pdy = sub2(sy2, *reinterpret_cast<const float2*>(&st->y[i]));
                        float2 d2 = fma2(pdy, pdy, mul2(pdx, pdx));
                        if (ND == 3) {
                            const float2 pdz =
                                sub2(sz2, *reinterpret_cast<const float2*>(&st->z[i]));
                            d2 = fma2(pdz, pdz, d2);
                        }
                        const int4 jj = *reinterpret_cast<const int4*>(&st->jc[i]);
                        if (jj.x >= mlo && jj.x < mhi && d2.x <= r2f) append(jj.x, jj.y);
                        if (i + 1 < nrel && jj.z >= mlo && jj.z < mhi && d2.y <= r2f)
                            append(jj.z, jj.w);
                    }
                    __syncwarp();
                }
            }
        }
    }
    const int stored = min(cnt, cap);
    if (active && (stored & 7)) flush(stored >> 3);  // the open chunk (tail entries unused)
    return cnt;
}

// Tiles of a fixed grid of resident blocks: each block takes the next 128-slot tile from
// ctr[0] until none is left (a closed gate then costs one short launch, and heavy tiles are
// spread over the blocks as they come); the last block to finish resets ctr[0..1] to zero for
// the next launch.
struct TileQueue {
    unsigned* ctr;
    __device__ __forceinline__ int next(int* slot) const {
        __syncthreads();  // every thread has read the previous tile
        if (threadIdx.x == 0) *slot = (int)atomicAdd(ctr, 1u);
        __syncthreads();
        return *slot;
    }
    __device__ __forceinline__ void done() const {
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(ctr + 1, 1u) == gridDim.x - 1) {
                ctr[0] = 0u;
                ctr[1] = 0u;
            }
        }
    }
};

// Fluid slots: fluid-fluid and fluid-wall lists, over the tiles of a TileQueue.
template <int ND>
__global__ void __launch_bounds__(128, 8) k_build_fluid_lists(
    GridDesc g, float cs, float m, float r2f, int nf, const float4* __restrict__ ftest,
    int fstride, const int* __restrict__ fskey, const int* __restrict__ fstart,
    const float4* __restrict__ wtest, const int* __restrict__ wskey,
    const int* __restrict__ wstart, unsigned* __restrict__ ff,
    int* __restrict__ ffc, int cap_ff, unsigned* __restrict__ fw, int* __restrict__ fwc,
    int cap_fw, int* __restrict__ err, const unsigned* __restrict__ gate, TileQueue q) {
    if (!gate_open(gate)) return;
    __shared__ SearchStage stage_all[4];
    __shared__ unsigned lbuf_all[kListChunk][128];
    __shared__ int tile_slot;
    SearchStage* st = &stage_all[threadIdx.x >> 5];
    unsigned* lbuf = &lbuf_all[0][threadIdx.x];
    const int ntiles = (nf + 127) / 128;
    for (int tile = q.next(&tile_slot); tile < ntiles; tile = q.next(&tile_slot)) {
        const int s = tile * 128 + threadIdx.x;
        const bool active = s < nf;
        const int si = active ? s : 0;
        const float4 ta = ftest[(size_t)si * fstride];
        int c[3];
        key_to_coords(fskey[si], g, c);
        const int n1 = warp_collect<ND>(g, cs, m, active, c, ta, fstart, fskey, ftest, fstride,
                                        r2f, st, lbuf, ff, nf, cap_ff, s);
        const int n2 = warp_collect<ND>(g, cs, m, active, c, ta, wstart, wskey, wtest, 1, r2f,
                                        st, lbuf, fw, nf, cap_fw, s);
        if (active) {
            ffc[s] = min(n1, cap_ff);
            fwc[s] = min(n2, cap_fw);
            if (n1 > cap_ff || n2 > cap_fw) atomicOr(err, TP_ERRBIT_CAPACITY);
        }
    }
    q.done();
}

// Wall slots: wall-fluid lists (the Adami gather), over the tiles of a TileQueue (most wall
// slots of a tank have no fluid in reach and finish their search at once).
template <int ND>
__global__ void __launch_bounds__(128, 8) k_build_wall_lists(
    GridDesc g, float cs, float m, float r2f, int nw, const float4* __restrict__ wtest,
    const int* __restrict__ wskey, const float4* __restrict__ ftest, int fstride,
    const int* __restrict__ fskey, const int* __restrict__ fstart, unsigned* __restrict__ wf,
    int* __restrict__ wfc, int cap_wf,
    int* __restrict__ err, const unsigned* __restrict__ gate, TileQueue q) {
    if (!gate_open(gate)) return;
    __shared__ SearchStage stage_all[4];
    __shared__ unsigned lbuf_all[kListChunk][128];
    __shared__ int tile_slot;
    SearchStage* st = &stage_all[threadIdx.x >> 5];
    unsigned* lbuf = &lbuf_all[0][threadIdx.x];
    const int ntiles = (nw + 127) / 128;
    for (int tile = q.next(&tile_slot); tile < ntiles; tile = q.next(&tile_slot)) {
        const int s = tile * 128 + threadIdx.x;
        const bool active = s < nw;
        const int si = active ? s : 0;
        const float4 ta = wtest[si];
        int c[3];
        key_to_coords(wskey[si], g, c);
        const int n1 = warp_collect<ND>(g, cs, m, active, c, ta, fstart, fskey, ftest, fstride,
                                        r2f, st, lbuf, wf, nw, cap_wf, s);
        if (active) {
            wfc[s] = min(n1, cap_wf);
            if (n1 > cap_wf) atomicOr(err, TP_ERRBIT_CAPACITY);
        }
    }
    q.done();
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
    if (g.org) {  // the same exact products from the origin table (FP64 throughput is scarce)
        const int base[3] = {0, g.n[0], g.n[0] + g.n[1]};
#pragma unroll
        for (int d = 0; d < ND; ++d) o[d] = (float)__dsub_rn(x[d], __ldg(g.org + base[d] + c[d]));
    } else {
#pragma unroll
        for (int d = 0; d < ND; ++d)
            o[d] = (float)__dsub_rn(x[d], __dmul_rn((double)(g.cmin[d] + c[d]), cs32));
    }
    return make_float4(o[0], o[1], o[2], (float)c[0]);
}

}  // namespace tp
