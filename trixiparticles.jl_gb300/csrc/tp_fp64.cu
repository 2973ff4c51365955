// tp_fp64.cu — plain FP64 drop-in form of the WCSPH right-hand side (sm_103a).
//
// Every physical quantity is Float64, as in the reference's Float64 GPU path.  Divisions the
// reference writes as `div_fast` use its CUDA Float64 definition x * fast_inv(y)
// (ext/TrixiParticlesCUDAExt.jl:12-32): approximate reciprocal `rcp.approx.ftz.f64` refined by
// one cubic iteration e = 1 - a r; e = e + e^2; r = r + e r (the method the reference takes from
// Oceananigans.jl PR 5140).  fast_inv(rho) of every particle is evaluated once per pass (pack:
// m_b / rho_b of the neighbour records; pair kernel: its own 1 / rho_a) and reused for every
// pair, which is bitwise the same as evaluating it per pair.  Plain `/` in the reference stays
// IEEE division here.
//
// Neighbour lists (tp_lists.cuh) are built with an FP32 distance on cell-relative offsets whose
// bound is widened by 1e-5 (FP32 rounding of d^2 is below 1e-6 relative).  At the start of every
// pair pass (fused into the pair kernel) the exact-list filter reduces them to the pairs with
// |x_a - x_b|^2 <= (2h)^2 decided in FP64 with explicitly rounded products and sums (no FMA
// contraction) wherever the FP32 test is not conclusive; the Adami kernel compacts its wall
// lists the same way.  The neighbour set is therefore the one the CPU computes, visited in the
// CPU's order.  The Cole EOS power and its inverse use repeated multiplication and Newton's
// method for the usual integer exponent (a few ulp of the correctly rounded values).
//
// On GB300 an FP64 FMA issues at 1/64 of the FP32 rate (about 20 SM cycles per warp
// instruction), so the pair kernel is FP64-throughput bound and the code spends FP32 and
// integer work freely to save FP64 instructions.
#include "tp_api_internal.h"
#include "tp_lists.cuh"

namespace tp {

__device__ __forceinline__ double fast_inv(double a) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(a));
    double e = fma(r, -a, 1.0);
    e = fma(e, e, e);
    return fma(e, r, r);
}

__device__ __forceinline__ double div_fast(double x, double y) { return x * fast_inv(y); }

// Pair distance r = sqrt(d2) for a normal d2 > 0, with few FP64 instructions: the approximate
// reciprocal square root y of `rsqrt.approx.ftz.f64` refined by one third-order Householder step
// for f(y) = y^-2 - d2 (e = 1 - d2 y^2, y' = y (1 + e/2 + 3 e^2 / 8), error O(e^3)), folded into
// r = d2 y' = t + t e (1/2 + 3 e / 8) with t = d2 y.  Within a few ulp of the rounded sqrt.
__device__ __forceinline__ double pair_distance(double d2) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d2));
    const double t = d2 * y;
    const double e = fma(-t, y, 1.0);
    return fma(t * e, fma(e, 0.375, 0.5), t);
}

template <int ND>
__device__ __forceinline__ double dist2_rn(double p0, double p1, double p2) {
    double d2 = __dadd_rn(__dmul_rn(p0, p0), __dmul_rn(p1, p1));
    if (ND == 3) d2 = __dadd_rn(d2, __dmul_rn(p2, p2));
    return d2;
}

// ------------------------------------------------------------------------------------------
// Pack: source particle i -> fluid record slot s.  The fluid EOS is evaluated here
// (compute_pressure!, weakly_compressible_sph/system.jl:426-438).
// ------------------------------------------------------------------------------------------
template <int ND>
struct Pack64 {
    const double* u;   // (ND, n) source order
    const double* v;   // (ND+1, n)
    const double* m;   // (n)
    const double* tu;  // optional: integrator registers (source order), moved with the state
    const double* tv;
    const int* id_in;
    double* tu_out;
    double* tv_out;
    int* id_out;
    double* m_out;
    double* xb_out;  // positions at the last rebuild (slot order), written on rebuild only
    float4* test;    // offsets against the reference cell (the cell of the last rebuild)
    double4_32a* pos;
    double4_32a* vel;
    // gather mode: {p S, S, A, 2 m alpha c h sg_c} with S = sg_c m / rho (the kernel
    // gradient's constant folded into the per-particle factors) and A = p_off + p - rho g.x
    // (the Adami sum term of a wall w is then A + rho g.x_w);
    // symmetric mode: {m, m / rho, 1 / rho, 2 m alpha c h};  1 / rho = fast_inv(rho)
    double4_32a* aux;
    int symmetric;
    const int* src_perm;  // kick! path: without a rebuild, slot s packs caller particle perm[s]
    GridDesc g;
    double cs32;
    Phys P;
    __device__ void operator()(int i, int s, int key, bool rebuild) const {
        if (!rebuild && src_perm) i = src_perm[s];
        double x[3] = {0, 0, 0}, w[4] = {0, 0, 0, 0};
#pragma unroll
        for (int d = 0; d < ND; ++d) x[d] = u[(size_t)i * ND + d];
#pragma unroll
        for (int d = 0; d <= ND; ++d) w[d] = v[(size_t)i * (ND + 1) + d];
        const double rho = w[ND];
        const double p = eos_pressure(rho, P, P.fluid_clip);
        const double mi = m[i];
        test[s] = test_record_in<ND>(x, g, cs32, key);  // every stage: the exact-list filter
        pos[s] = make_double4_32a(x[0], x[1], ND == 3 ? x[2] : 0.0, p);
        vel[s] = make_double4_32a(w[0], w[1], ND == 3 ? w[2] : 0.0, rho);
        const double ir = fast_inv(rho);
        if (symmetric) {
            aux[s] = make_double4_32a(mi, mi * ir, ir, mi * P.visc_k2);
        } else {
            const double S = P.sg_c * (mi * ir);
            double gx = P.g[0] * x[0] + P.g[1] * x[1];
            if (ND == 3) gx += P.g[2] * x[2];
            aux[s] = make_double4_32a(p * S, S, fma(-rho, gx, P.p_off + p), mi * P.visc_k2s);
        }
        if (rebuild && xb_out) {
#pragma unroll
            for (int d = 0; d < ND; ++d) xb_out[(size_t)s * ND + d] = x[d];
        }
        if (tu_out) {
#pragma unroll
            for (int d = 0; d < ND; ++d) tu_out[(size_t)s * ND + d] = tu[(size_t)i * ND + d];
#pragma unroll
            for (int d = 0; d <= ND; ++d)
                tv_out[(size_t)s * (ND + 1) + d] = tv[(size_t)i * (ND + 1) + d];
            id_out[s] = id_in[i];
            m_out[s] = mi;
        }
    }
};

// Positions only (p = 0): neighbour-count diagnostics.
template <int ND>
struct PackPos64 {
    const double* u;
    double4_32a* pos;
    __device__ void operator()(int i, int s, int, bool) const {
        double x[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < ND; ++d) x[d] = u[(size_t)i * ND + d];
        pos[s] = make_double4_32a(x[0], x[1], x[2], 0.0);
    }
};

// Wall records (setup): FP64 {x, y, z, m} and the FP32 test record.
template <int ND>
struct PackWall64 {
    const double* x;
    const double* m;
    double4_32a* pos;
    float4* test;
    GridDesc g;
    double cs32;
    __device__ void operator()(int i, int s, int key, bool) const {
        double y[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < ND; ++d) y[d] = x[(size_t)i * ND + d];
        pos[s] = make_double4_32a(y[0], y[1], y[2], m[i]);
        test[s] = test_record_in<ND>(y, g, cs32, key);
    }
};

// ------------------------------------------------------------------------------------------
// Adami pressure extrapolation (dummy_particles.jl:489-569, 586-606, 637-672): one lane per
// wall slot gathers its fluid neighbours in PointNeighbors order.
// ------------------------------------------------------------------------------------------
// ------------------------------------------------------------------------------------------
// Fused fluid pair kernel: fluid-fluid then fluid-wall interactions of one fluid slot
// (weakly_compressible_sph/rhs.jl:30-124), plus gravity (semidiscretization.jl:701-731), then
// either the dv write (kick!) or the CarpenterKennedy2N54 register update of the slot.
// ------------------------------------------------------------------------------------------
struct Update64 {
    double* dv;        // kick mode: dv_ode in source order (indexed by perm)
    const int* perm;
    // integrate mode (slot order, in place on the state written by this stage's pack):
    double* u_out;
    double* v_out;
    double* tu;
    double* tv;
    // displacement check of the next stage (optional): positions of the last rebuild (slot
    // order) and the gate word that collects the largest squared displacement
    const double* xb;
    unsigned* gate_next;
    double A, B, dt;
    int first;
};

// kick!: dv write in caller order; integrator: CarpenterKennedy2N54 stage of slot s,
// tmp = A*tmp + dt*k ; y = y + B*tmp (du = v at stage start).
template <int ND, bool INTEGRATE>
__device__ __forceinline__ void stage_update(int s, const double4_32a& pa, const double4_32a& va,
                                             const double (&k)[4], const Update64& U) {
    if (!INTEGRATE) {
        const int i = U.perm[s];
#pragma unroll
        for (int d = 0; d <= ND; ++d) U.dv[(size_t)i * (ND + 1) + d] = k[d];
    } else {
        const double va_arr[4] = {va.x, va.y, ND == 3 ? va.z : va.w, va.w};
        const double xa_arr[3] = {pa.x, pa.y, pa.z};
#pragma unroll
        for (int d = 0; d <= ND; ++d) {
            const double kv = k[d];
            double tv = U.first ? U.dt * kv : fma(U.dt, kv, U.A * U.tv[(size_t)s * (ND + 1) + d]);
            U.tv[(size_t)s * (ND + 1) + d] = tv;
            U.v_out[(size_t)s * (ND + 1) + d] = fma(U.B, tv, va_arr[d]);
        }
        double un[ND];
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const double ku = va_arr[d];
            double tu = U.first ? U.dt * ku : fma(U.dt, ku, U.A * U.tu[(size_t)s * ND + d]);
            U.tu[(size_t)s * ND + d] = tu;
            un[d] = fma(U.B, tu, xa_arr[d]);
            U.u_out[(size_t)s * ND + d] = un[d];
        }
        if (U.gate_next)
            gate_max_displacement(U.gate_next, displacement2<ND>(un, U.xb + (size_t)s * ND));
    }
}

// Exact pair lists of this stage: the skin list of every fluid slot reduced to the pairs with
// |x_a - x_b|^2 <= (2h)^2 (FP64, explicitly rounded products and sums), self excluded, in list
// (PointNeighbors) order.  The FP32 distance on the cell-relative offsets decides every candidate
// whose d^2 lies further than 1e-5 relative from the bound (its rounding error is below 1e-6
// relative); only candidates inside that band are decided from the FP64 records.  FP64
// arithmetic runs at 1/64 of the FP32 rate on this GPU, so removing the ~25 % of listed
// candidates that lie in the skin shell from the FP64 pair loop is worth an extra pass.
template <int ND>
__device__ __forceinline__ int filter_list(int s, int n_rows, float4 ta, const float4* off,
                                           float lo2, float hi2, float zero2, double sr2,
                                           double az2, const double4_32a& pa,
                                           const float4* __restrict__ test,
                                           const double4_32a* __restrict__ pos,
                                           const unsigned* __restrict__ list,
                                           int cnt, int skip, unsigned* out,
                                           unsigned* lbuf) {
    // skip: 0 keep all (walls), 1 drop self (fluid, gather mode), 2 keep the pairs that s owns
    // (fluid, symmetric mode: the owner of {s, b} is the lower slot when s + b is odd and the
    // higher one when it is even; measured on GB300 this balances the lanes better than a hashed
    // owner, whose scattered accesses cost more than its balance gains)
    int n = 0;
    // exact list in the chunked layout of the skin lists, whole chunks written from the lane's
    // column of the block buffer (entry r of the open chunk at lbuf[r * blockDim.x])
    const int bs = blockDim.x;
    auto flush = [&](int q) {
        uint4* dst = reinterpret_cast<uint4*>(out + list_at(q * kListChunk, n_rows, s));
        dst[0] = make_uint4(lbuf[0], lbuf[bs], lbuf[2 * bs], lbuf[3 * bs]);
        dst[1] = make_uint4(lbuf[4 * bs], lbuf[5 * bs], lbuf[6 * bs], lbuf[7 * bs]);
    };
    auto test_one = [&](unsigned e, const float4& cb) {
        const int b = (int)(e & kSlotMask);
        if (b == s && skip != 0) return;
        if (skip == 2 && ((b > s) != (((s ^ b) & 1) != 0))) return;
        float p0, p1, p2;
        const float d2f = pair_diff<ND>(ta, off, e, cb, p0, p1, p2);
        bool acc = d2f <= lo2;
        if ((!acc && d2f <= hi2) || (acc && d2f < zero2)) {
            // decided in FP64: the support bound, and the zero-distance skip of rhs.jl:27-28
            // (distance < sqrt(eps((2h)^2)), tested as d^2 < eps((2h)^2)) for near-coincident pairs
            const double4_32a pb = pos[b];
            const double d2 = dist2_rn<ND>(pa.x - pb.x, pa.y - pb.y, ND == 3 ? pa.z - pb.z : 0.0);
            acc = d2 <= sr2 && !(d2 < az2);
        }
        if (acc) {
            lbuf[(n & 7) * bs] = (unsigned)b;
            if ((n & 7) == 7) flush(n >> 3);
            ++n;
        }
    };
    // four candidates' entries and records in flight at a time (the pass is gather-latency
    // bound); tested in list order
    int k = 0;
    for (; k + 4 <= cnt; k += 4) {
        const uint4 q = list_quad(list, k, n_rows, s);
        const unsigned e[4] = {q.x, q.y, q.z, q.w};
        float4 cb[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) cb[j] = test[e[j] & kSlotMask];
#pragma unroll
        for (int j = 0; j < 4; ++j) test_one(e[j], cb[j]);
    }
    for (; k < cnt; ++k) {
        const unsigned e = list[list_at(k, n_rows, s)];
        test_one(e, test[e & kSlotMask]);
    }
    if (n & 7) flush(n >> 3);  // the open chunk (tail entries unused)
    return n;
}

template <int ND>
__global__ void __launch_bounds__(256) k_filter64(
    double sr2, double az2, float cs, float lo2, float hi2, float zero2, int nf,
    const float4* __restrict__ ftest,
    const double4_32a* __restrict__ fpos, const unsigned* __restrict__ ff,
    const int* __restrict__ ffc, const unsigned* __restrict__ fw, const int* __restrict__ fwc,
    const float4* __restrict__ wtest, const double4_32a* __restrict__ wpos, int* __restrict__ eff,
    int* __restrict__ effc, int* __restrict__ efw, int* __restrict__ efwc, int half) {
    __shared__ float4 off[kOffsetCodes];
    __shared__ unsigned lbuf_all[kListChunk][256];
    fill_offset_table(off, cs);
    unsigned* lbuf = &lbuf_all[0][threadIdx.x];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    const float4 ta = ftest[s];
    const double4_32a pa = fpos[s];
    effc[s] = filter_list<ND>(s, nf, ta, off, lo2, hi2, zero2, sr2, az2, pa, ftest, fpos, ff,
                              ffc[s], half ? 2 : 1, (unsigned*)eff, lbuf);
    efwc[s] = filter_list<ND>(s, nf, ta, off, lo2, hi2, zero2, sr2, az2, pa, wtest, wpos, fw,
                              fwc[s], 0, (unsigned*)efw, lbuf);
}

// Pair terms of rhs.jl:81-117 (pressure, Monaghan viscosity, continuity, Molteni-Colagrossi
// diffusion), FP64 throughout, written for the slow FP64 pipe with the identities that follow
// from grad W_ab = sg * x_ab (sg = sg_c (1 - q/2)^3, kernel_deriv_div_r_unsafe):
//   pressure + viscosity: dv_a += (c_p + c_v) sg x_ab, one scalar for both terms;
//   continuity: v_ab . grad W = sg (v_ab . x_ab), the dot product the viscosity switch needs;
//   diffusion: psi_ab . grad W = 2 (rho_a - rho_b) / r^2 (x_ab . sg x_ab) = 2 (rho_a - rho_b) sg;
//   Monaghan: mu / rho_mean from one reciprocal of (r^2 + eps h^2) rho_mean;
//   1 / (rho_a rho_b) and m_b / rho_b from the per-particle fast_inv(rho) of the pack;
//   the constant sg_c folded into the neighbour records (S_b = sg_c m_b / rho_b, p_b S_b,
//   2 m_b alpha c h sg_c), so the pressure factor is one FMA and sg is t^3 alone;
//   r from d^2 by pair_distance; the zero-distance skip `distance < sqrt(eps((2h)^2))` (rhs.jl:27-28)
//   tested as d^2 < eps((2h)^2).
// Each term equals the reference's expression up to a few ulp of rounding.
__device__ __forceinline__ double monaghan_coef(const Phys& P, const double4_32a& ab, double rho_b,
                                                double vr, double d2, double rho_sum) {
    // sg_c m_b (alpha c mu + beta mu^2) / rho_mean, mu = h vr / (r^2 + eps h^2),
    // rho_mean = rho_sum / 2 (vr < 0); ab.w = 2 m_b alpha c h sg_c, ab.y rho_b = sg_c m_b
    const double den = d2 + P.visc_eps_h2;
    const double R = fast_inv(den * rho_sum);
    if (P.beta == 0.0) return ab.w * vr * R;
    const double mu = (P.visc_h * vr) * (rho_sum * R);
    return ((ab.y * rho_b) * mu) * (P.alpha_c + P.beta * mu) * (2.0 * den * R);
}

// The support test is the exact-list filter's (FP32 on the cell-relative offsets outside a 1e-5
// band around (2h)^2, the CPU's explicitly rounded FP64 test inside it), run first over the whole
// skin list: the accepted fluid neighbours are compacted into the wall's exact list (chunked
// layout, written and read back by the same thread) and the FP64 loop walks only those, so the
// lanes of a warp stay busy on the FP64 pipe (wall particles deep in the wall layers have few
// fluid neighbours).  Distances of accepted pairs are formed with FMAs.
// FOLD (gather pair mode): the fluid records carry A_f = p_off + p_f - rho_f g.x_f, so the sum
// term p_off + p_f + g.(rho_f (x_w - x_f)) is fma(rho_f, g.x_w, A_f), and the kernel's norm is
// applied once to the sums (their ratio does not depend on it).
template <int ND, bool FOLD>
__global__ void __launch_bounds__(256) k_adami64(Phys P, int nw,
                                                 const double4_32a* __restrict__ wpos,
                                                 const float4* __restrict__ wtest,
                                                 const unsigned* __restrict__ wf,
                                                 const int* __restrict__ wfc,
                                                 double4_32a* __restrict__ wstate,
                                                 double* __restrict__ wvol,
                                                 const double4_32a* __restrict__ fpos,
                                                 const double4_32a* __restrict__ fvel,
                                                 const double4_32a* __restrict__ faux,
                                                 const float4* __restrict__ ftest, float cs,
                                                 float lo2, float hi2, unsigned* ewf) {
    __shared__ float4 off[kOffsetCodes];
    __shared__ unsigned lbuf_all[kListChunk][256];
    fill_offset_table(off, cs);
    unsigned* lbuf = &lbuf_all[0][threadIdx.x];
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    const double4_32a xw = wpos[w];
    const float4 tw = wtest[w];
    // exact list of the wall: d^2 <= (2h)^2, zero distance included (no skip in the Adami sum)
    const int n = filter_list<ND>(w, nw, tw, off, lo2, hi2, -1.0f, P.sr2, -1.0, xw, ftest, fpos,
                                  wf, wfc[w], 0, ewf, lbuf);
    double gxw = P.g[0] * xw.x + P.g[1] * xw.y;
    if (ND == 3) gxw += P.g[2] * xw.z;
    const double two_hinv = 2.0 * P.h_inv;
    double Ps = 0.0, V = 0.0;
    uint4 lq;  // the exact-list quad holding entry k
    for (int k = 0; k < n; ++k) {
        const int b = (int)list_next_rw(ewf, k, nw, w, lq);
        const double4_32a xb = fpos[b];
        const double pd0 = xw.x - xb.x, pd1 = xw.y - xb.y;
        const double pd2 = (ND == 3) ? xw.z - xb.z : 0.0;
        double d2 = pd0 * pd0 + pd1 * pd1;
        if (ND == 3) d2 += pd2 * pd2;
        const double r = d2 > 0.0 ? pair_distance(d2) : 0.0;
        const double rho_f = fvel[b].w;
        double sum;
        if (FOLD) {
            sum = fma(rho_f, gxw, faux[b].z);
        } else {
            double hp = P.g[0] * (rho_f * pd0) + P.g[1] * (rho_f * pd1);
            if (ND == 3) hp += P.g[2] * (rho_f * pd2);
            sum = (P.p_off + xb.w) + hp;
        }
        double W = 0.0;
        if (r < P.two_h) {  // (1 - q/2)^4 (2q + 1), q = r / h
            const double t = fma(-r, P.half_hinv, 1.0);
            const double t2 = t * t;
            W = FOLD ? (t2 * t2) * fma(r, two_hinv, 1.0)
                     : (P.wc2_norm * (t2 * t2)) * fma(r, two_hinv, 1.0);
        }
        Ps = fma(sum, W, Ps);
        V += W;
    }
    if (FOLD) {
        const double Vn = P.wc2_norm * V;
        Ps = Vn > 2.220446049250313e-16 ? Ps / V : P.wc2_norm * Ps;
        V = Vn;
    } else if (V > 2.220446049250313e-16) {
        Ps = Ps / V;
    }
    if (P.wall_clip) Ps = (Ps != Ps || Ps > 0.0) ? Ps : 0.0;
    const double rho_w = eos_inverse(Ps, P);
    const double ir_w = fast_inv(rho_w);
    if (FOLD) {
        const double S = P.sg_c * (xw.w * ir_w);
        wstate[w] = make_double4_32a(Ps, rho_w, Ps * S, S);  // {p, rho, p S, S = sg_c m/rho}
    } else {
        wstate[w] = make_double4_32a(Ps, rho_w, ir_w, xw.w * ir_w);  // {p, rho, 1/rho, m/rho}
    }
    wvol[w] = V;
}


// Skin lists in, exact lists of this stage out (the filter fused into the gather pair kernel).
struct Filter64 {
    float cs, lo2, hi2, zero2;
    const float4* ftest;
    const float4* wtest;
    const unsigned* ff;
    const int* ffc;
    const unsigned* fw;
    const int* fwc;
    int* eff;  // written and read back by the same thread: no restrict, no read-only path
    int* efw;
};

// The gather pass first filters its slot's skin lists into exact lists (the same filter_list as
// k_filter64), then walks them.  Fused, the filter's gathers and FP32 tests of some warps run
// under the FP64 pair arithmetic of others instead of in a latency-bound pass of their own.
template <int ND, bool INTEGRATE>
__global__ void __launch_bounds__(256) k_pair64(Phys P, int nf,
                                                const double4_32a* __restrict__ fpos,
                                                const double4_32a* __restrict__ fvel,
                                                const double4_32a* __restrict__ faux,
                                                Filter64 F,
                                                const double4_32a* __restrict__ wpos,
                                                const double4_32a* __restrict__ wstate,
                                                Update64 U) {
    __shared__ float4 off[kOffsetCodes];
    __shared__ unsigned lbuf_all[kListChunk][256];
    fill_offset_table(off, F.cs);
    unsigned* lbuf = &lbuf_all[0][threadIdx.x];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    const double4_32a pa = fpos[s];
    const double4_32a va = fvel[s];
    const float4 ta = F.ftest[s];
    const int nff = filter_list<ND>(s, nf, ta, off, F.lo2, F.hi2, F.zero2, P.sr2, P.az2, pa,
                                    F.ftest, fpos, F.ff, F.ffc[s], 1, (unsigned*)F.eff, lbuf);
    const int nfw = filter_list<ND>(s, nf, ta, off, F.lo2, F.hi2, F.zero2, P.sr2, P.az2, pa,
                                    F.wtest, wpos, F.fw, F.fwc[s], 0, (unsigned*)F.efw, lbuf);
    const unsigned* eff = (const unsigned*)F.eff;
    const unsigned* efw = (const unsigned*)F.efw;
    uint4 lq;  // the exact-list quad holding entry k
    const double p_a = pa.w, rho_a = va.w, nia = -fast_inv(rho_a);  // the pack's 1 / rho

    // ---- fluid-fluid ----
    double dv0 = 0.0, dv1 = 0.0, dv2 = 0.0, drho = 0.0;
    for (int k = 0; k < nff; ++k) {
        const int b = (int)list_next_rw(eff, k, nf, s, lq);
        const double4_32a pb = fpos[b];
        const double pd0 = pa.x - pb.x, pd1 = pa.y - pb.y;
        const double pd2 = (ND == 3) ? pa.z - pb.z : 0.0;
        double d2 = pd0 * pd0 + pd1 * pd1;
        if (ND == 3) d2 += pd2 * pd2;
        const double r = pair_distance(d2);  // d2 >= eps((2h)^2): the filter dropped closer pairs
        const double t = fma(-r, P.half_hinv, 1.0);
        const double t3 = (t * t) * t;  // grad W_ab = sg_c t^3 x_ab, sg_c folded into ab
        const double4_32a vb = fvel[b];
        const double4_32a ab = faux[b];  // {p_b S_b, S_b, A_b, 2 m_b alpha c h sg_c}
        const double vd0 = va.x - vb.x, vd1 = va.y - vb.y;
        const double vd2 = (ND == 3) ? va.z - vb.z : 0.0;
        double vr = vd0 * pd0 + vd1 * pd1;
        if (ND == 3) vr += vd2 * pd2;
        // -sg_c m_b (p_a + p_b) / (rho_a rho_b) = -(p_a S_b + p_b S_b) / rho_a
        double c = nia * fma(p_a, ab.y, ab.x);
        if (P.visc && vr < 0.0) c += monaghan_coef(P, ab, vb.w, vr, d2, rho_a + vb.w);
        c *= t3;
        dv0 += c * pd0;
        dv1 += c * pd1;
        if (ND == 3) dv2 += c * pd2;
        // continuity (rho_a / rho_b) m_b v_ab . grad W  +  diffusion m_b / rho_b psi . grad W
        const double dd = P.diff ? P.diff2 * (rho_a - vb.w) : 0.0;
        drho += (ab.y * t3) * fma(rho_a, vr, dd);
    }

    // ---- fluid-wall (wall viscosity = nothing, no density diffusion, wall velocity 0) ----
    double ew0 = 0.0, ew1 = 0.0, ew2 = 0.0, erho = 0.0;
    for (int k = 0; k < nfw; ++k) {
        const int b = (int)list_next_rw(efw, k, nf, s, lq);
        const double4_32a pb = wpos[b];
        const double pd0 = pa.x - pb.x, pd1 = pa.y - pb.y;
        const double pd2 = (ND == 3) ? pa.z - pb.z : 0.0;
        double d2 = pd0 * pd0 + pd1 * pd1;
        if (ND == 3) d2 += pd2 * pd2;
        const double r = pair_distance(d2);
        const double t = fma(-r, P.half_hinv, 1.0);
        const double t3 = (t * t) * t;
        const double4_32a sb = wstate[b];  // {p, rho, p S, S = sg_c m / rho}
        const double c = (nia * fma(p_a, sb.w, sb.z)) * t3;
        ew0 += c * pd0;
        ew1 += c * pd1;
        if (ND == 3) ew2 += c * pd2;
        double vx = va.x * pd0 + va.y * pd1;
        if (ND == 3) vx += va.z * pd2;
        erho += (rho_a * sb.w) * (t3 * vx);
    }

    // dv = ((0 + S_ff) + S_fw) + g ;  drho = S_ff + S_fw
    double k[4];
    k[0] = (dv0 + ew0) + P.g[0];
    k[1] = (dv1 + ew1) + P.g[1];
    k[2] = (ND == 3) ? (dv2 + ew2) + P.g[2] : 0.0;
    k[ND] = drho + erho;
    stage_update<ND, INTEGRATE>(s, pa, va, k, U);
}

// Symmetric pair pass: every fluid-fluid pair once, at its owner a (the exact half list holds
// the pairs a owns).  b receives the terms it would evaluate itself -- with x_ba = -x_ab,
// v_ba = -v_ab, grad W_ba = -grad W_ab the shared factors (sg, p_a + p_b, the Monaghan
// reciprocal, v_ab . x_ab, rho_a - rho_b) are evaluated once -- through FP64 atomic adds into
// its accumulator {dv, drho}; a adds its own sum once at the end.  Lanes of a warp start their
// walk at different points of their lists, so that the atomic adds of neighbouring lanes (whose
// candidate sequences are nearly the same) do not hit the same particle at the same time.
// Fluid-wall pairs stay one-sided.  k_update64 then applies gravity and the stage.
template <int ND>
__global__ void __launch_bounds__(256) k_pair64s(Phys P, int nf,
                                                 const double4_32a* __restrict__ fpos,
                                                 const double4_32a* __restrict__ fvel,
                                                 const double4_32a* __restrict__ faux,
                                                 const int* __restrict__ eff,
                                                 const int* __restrict__ effc,
                                                 const int* __restrict__ efw,
                                                 const int* __restrict__ efwc,
                                                 const double4_32a* __restrict__ wpos,
                                                 const double4_32a* __restrict__ wstate,
                                                 double* __restrict__ acc) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    const double4_32a pa = fpos[s];
    const double4_32a va = fvel[s];
    const double4_32a aa = faux[s];
    const double p_a = pa.w, rho_a = va.w, m_a = aa.x, vol_a = aa.y, ia = aa.z;

    double dv0 = 0.0, dv1 = 0.0, dv2 = 0.0, drho = 0.0;
    const int nff = effc[s];
    int k = (int)(((unsigned)(threadIdx.x & 31) * (unsigned)nff) >> 5);
    for (int it = 0; it < nff; ++it, ++k) {
        if (k == nff) k = 0;
        const int b = eff[list_at(k, nf, s)];
        const double4_32a pb = fpos[b];
        const double pd0 = pa.x - pb.x, pd1 = pa.y - pb.y;
        const double pd2 = (ND == 3) ? pa.z - pb.z : 0.0;
        double d2 = pd0 * pd0 + pd1 * pd1;
        if (ND == 3) d2 += pd2 * pd2;
        const double r = pair_distance(d2);
        const double t = fma(-r, P.half_hinv, 1.0);
        const double sg = P.sg_c * ((t * t) * t);
        const double4_32a vb = fvel[b];
        const double4_32a ab = faux[b];
        const double rho_b = vb.w;
        const double vd0 = va.x - vb.x, vd1 = va.y - vb.y;
        const double vd2 = (ND == 3) ? va.z - vb.z : 0.0;
        double vr = vd0 * pd0 + vd1 * pd1;
        if (ND == 3) vr += vd2 * pd2;
        const double Pab = p_a + pb.w;
        // a: -m_b (p_a+p_b)/(rho_a rho_b) grad W_ab ; b: -m_a (p_a+p_b)/(rho_a rho_b) grad W_ba
        double ca = -(ab.y * ia) * Pab;
        double cb = (vol_a * ab.z) * Pab;
        if (P.visc && vr < 0.0) {
            const double den = d2 + P.visc_eps_h2;
            const double rm = 0.5 * (rho_a + rho_b);
            const double R = fast_inv(den * rm);
            if (P.beta == 0.0) {
                const double w = vr * R;
                ca += (ab.x * P.visc_k) * w;
                cb -= (m_a * P.visc_k) * w;
            } else {
                const double mu = (P.visc_h * vr) * (rm * R);
                const double w = mu * (P.alpha_c + P.beta * mu) * (den * R);
                ca += ab.x * w;
                cb -= m_a * w;
            }
        }
        ca *= sg;
        cb *= sg;
        dv0 += ca * pd0;
        dv1 += ca * pd1;
        if (ND == 3) dv2 += ca * pd2;
        const double svr = sg * vr;
        drho += (rho_a * ab.y) * svr;
        double br = (rho_b * vol_a) * svr;
        if (P.diff) {
            const double dd = (rho_a - rho_b) * (sg * P.diff2);
            drho += ab.y * dd;
            br -= vol_a * dd;
        }
        double* ab4 = acc + (size_t)b * 4;
        atomicAdd(ab4 + 0, cb * pd0);
        atomicAdd(ab4 + 1, cb * pd1);
        if (ND == 3) atomicAdd(ab4 + 2, cb * pd2);
        atomicAdd(ab4 + 3, br);
    }

    const int nfw = efwc[s];
    for (int kw = 0; kw < nfw; ++kw) {
        const int b = efw[list_at(kw, nf, s)];
        const double4_32a pb = wpos[b];
        const double pd0 = pa.x - pb.x, pd1 = pa.y - pb.y;
        const double pd2 = (ND == 3) ? pa.z - pb.z : 0.0;
        double d2 = pd0 * pd0 + pd1 * pd1;
        if (ND == 3) d2 += pd2 * pd2;
        const double r = pair_distance(d2);
        const double t = fma(-r, P.half_hinv, 1.0);
        const double sg = P.sg_c * ((t * t) * t);
        const double4_32a sb = wstate[b];
        const double c = (-(sb.w * ia) * (p_a + sb.x)) * sg;
        dv0 += c * pd0;
        dv1 += c * pd1;
        if (ND == 3) dv2 += c * pd2;
        double vx = va.x * pd0 + va.y * pd1;
        if (ND == 3) vx += va.z * pd2;
        drho += (rho_a * sb.w) * (sg * vx);
    }
    double* a4 = acc + (size_t)s * 4;
    atomicAdd(a4 + 0, dv0);
    atomicAdd(a4 + 1, dv1);
    if (ND == 3) atomicAdd(a4 + 2, dv2);
    atomicAdd(a4 + 3, drho);
}

// Gravity + stage update (or the kick! write) from the symmetric pass's accumulators, which are
// cleared for the next pass.
template <int ND, bool INTEGRATE>
__global__ void __launch_bounds__(256) k_update64(Phys P, int nf,
                                                  const double4_32a* __restrict__ fpos,
                                                  const double4_32a* __restrict__ fvel,
                                                  double* __restrict__ acc, Update64 U) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    double4_32a a4 = *(const double4_32a*)(acc + (size_t)s * 4);
    *(double4_32a*)(acc + (size_t)s * 4) = make_double4_32a(0.0, 0.0, 0.0, 0.0);
    double k[4];
    k[0] = a4.x + P.g[0];
    k[1] = a4.y + P.g[1];
    k[2] = (ND == 3) ? a4.z + P.g[2] : 0.0;
    k[ND] = a4.w;
    stage_update<ND, INTEGRATE>(s, fpos[s], fvel[s], k, U);
}

// Neighbour counting (diagnostics): fluid-fluid, fluid-wall for fluid slots, or wall-fluid.
template <int ND>
__global__ void k_count64(GridDesc g, double sr2, int n, const double4_32a* __restrict__ qpos,
                          const int* __restrict__ qskey, const int* __restrict__ qperm,
                          const double4_32a* __restrict__ npos, const int* __restrict__ nstart,
                          int* __restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double4_32a pa = qpos[s];
    int c[3];
    key_to_coords(qskey[s], g, c);
    int cnt = 0;
    const int zlo = (ND == 3) ? -1 : 0, zhi = (ND == 3) ? 1 : 0;
    for (int dz = zlo; dz <= zhi; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            const int row = (c[0] - 1) + g.n[0] * ((c[1] + dy) + g.n[1] * (c[2] + dz));
            for (int b = nstart[row]; b < nstart[row + 3]; ++b) {
                const double4_32a pb = npos[b];
                const double d2 = dist2_rn<ND>(pa.x - pb.x, pa.y - pb.y,
                                               (ND == 3) ? pa.z - pb.z : 0.0);
                cnt += (d2 <= sr2);
            }
        }
    out[qperm[s]] = cnt;
}

// ------------------------------------------------------------------------------------------
// Host launchers
// ------------------------------------------------------------------------------------------
namespace {
inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }
}  // namespace

template <int ND>
static void pack_fluid64(tp_handle* h, const double* u, const double* v, const double* m,
                         const PhysState* src, PhysState* dst, const unsigned* gate) {
    Pack64<ND> pk{};
    pk.u = u;
    pk.v = v;
    pk.m = m;
    pk.src_perm = (!src && gate) ? h->f_perm : nullptr;
    if (src) {
        pk.tu = src->tu;
        pk.tv = (const double*)src->tv;
        pk.id_in = src->id;
        pk.tu_out = dst->tu;
        pk.tv_out = (double*)dst->tv;
        pk.id_out = dst->id;
        pk.m_out = (double*)dst->m;
    }
    pk.xb_out = h->x_build;
    pk.test = h->f_test;
    pk.pos = (double4_32a*)h->f_pos;
    pk.vel = (double4_32a*)h->f_vel;
    pk.aux = (double4_32a*)h->f_aux;
    pk.symmetric = h->pair_mode == TP_PAIR_SYMMETRIC;
    pk.g = h->grid;
    pk.cs32 = (double)(float)h->grid.cs;
    pk.P = h->phys;
    const int n = (int)h->cfg.n_fluid;
    k_rank_pack<<<nblk(n, 256), 256, 0, h->stream>>>(h->f_tmp, h->f_key, h->f_start, n, h->f_perm,
                                                      h->f_skey, pk, gate);
}

void fp64_pack(tp_handle* h, const double* u, const double* v, const double* m,
               const PhysState* src, PhysState* dst, const unsigned* gate) {
    if (h->cfg.n_fluid == 0) return;
    if (h->cfg.ndims == 2)
        pack_fluid64<2>(h, u, v, m, src, dst, gate);
    else
        pack_fluid64<3>(h, u, v, m, src, dst, gate);
}

void fp64_pack_pos(tp_handle* h, const double* u) {
    const int n = (int)h->cfg.n_fluid;
    if (n == 0) return;
    if (h->cfg.ndims == 2) {
        PackPos64<2> pk{u, (double4_32a*)h->f_pos};
        k_rank_pack<<<nblk(n, 256), 256, 0, h->stream>>>(h->f_tmp, h->f_key, h->f_start, n,
                                                          h->f_perm, h->f_skey, pk);
    } else {
        PackPos64<3> pk{u, (double4_32a*)h->f_pos};
        k_rank_pack<<<nblk(n, 256), 256, 0, h->stream>>>(h->f_tmp, h->f_key, h->f_start, n,
                                                          h->f_perm, h->f_skey, pk);
    }
}

void fp64_pack_wall(tp_handle* h, const double* x, const double* m) {
    const int n = (int)h->cfg.n_wall;
    if (n == 0) return;
    const double cs32 = (double)(float)h->grid.cs;
    if (h->cfg.ndims == 2) {
        PackWall64<2> pk{x, m, (double4_32a*)h->w_pos, h->w_test, h->grid, cs32};
        k_rank_pack<<<nblk(n, 256), 256, 0, h->stream>>>(h->w_tmp, h->w_key, h->w_start, n,
                                                          h->w_perm, h->w_skey, pk);
    } else {
        PackWall64<3> pk{x, m, (double4_32a*)h->w_pos, h->w_test, h->grid, cs32};
        k_rank_pack<<<nblk(n, 256), 256, 0, h->stream>>>(h->w_tmp, h->w_key, h->w_start, n,
                                                          h->w_perm, h->w_skey, pk);
    }
}

void fp64_adami(tp_handle* h) {
    const int nw = (int)h->cfg.n_wall;
    if (nw == 0) return;
    const bool fold = h->pair_mode != TP_PAIR_SYMMETRIC;
    const double sr2 = h->phys.sr2;
    const float cs = (float)h->grid.cs, lo2 = (float)(sr2 * (1.0 - 1e-5)),
                hi2 = (float)(sr2 * (1.0 + 1e-5));
    auto run = [&](auto ndc, auto foldc) {
        constexpr int ND = decltype(ndc)::value;
        k_adami64<ND, decltype(foldc)::value><<<nblk(nw, h->pair_block), h->pair_block, 0,
                                                 h->stream>>>(
            h->phys, nw, (const double4_32a*)h->w_pos, h->w_test, h->l_wf, h->c_wf,
            (double4_32a*)h->w_state, h->w_vol, (const double4_32a*)h->f_pos,
            (const double4_32a*)h->f_vel, (const double4_32a*)h->f_aux, h->f_test, cs, lo2, hi2,
            (unsigned*)h->e_wf);
    };
    if (h->cfg.ndims == 2) {
        if (fold) run(std::integral_constant<int, 2>{}, std::true_type{});
        else run(std::integral_constant<int, 2>{}, std::false_type{});
    } else {
        if (fold) run(std::integral_constant<int, 3>{}, std::true_type{});
        else run(std::integral_constant<int, 3>{}, std::false_type{});
    }
}

template <int ND, bool INTEG>
static void launch_pair64(tp_handle* h, const Update64& U) {
    const int nf = (int)h->cfg.n_fluid;
    const double sr2 = h->phys.sr2;
    const bool sym = h->pair_mode == TP_PAIR_SYMMETRIC;
    const float lo2 = (float)(sr2 * (1.0 - 1e-5)), hi2 = (float)(sr2 * (1.0 + 1e-5));
    const float zero2 = (float)(sr2 * 1e-6);
    if (sym) {
        k_filter64<ND><<<nblk(nf, 256), 256, 0, h->stream>>>(
            sr2, h->phys.az2, (float)h->grid.cs, lo2, hi2, zero2, nf, h->f_test,
            (const double4_32a*)h->f_pos, h->l_ff, h->c_ff, h->l_fw, h->c_fw, h->w_test,
            (const double4_32a*)h->w_pos, h->e_ff, h->ec_ff, h->e_fw, h->ec_fw, 1);
        k_pair64s<ND><<<nblk(nf, h->pair_block), h->pair_block, 0, h->stream>>>(
            h->phys, nf, (const double4_32a*)h->f_pos, (const double4_32a*)h->f_vel,
            (const double4_32a*)h->f_aux, h->e_ff, h->ec_ff, h->e_fw, h->ec_fw,
            (const double4_32a*)h->w_pos, (const double4_32a*)h->w_state, h->acc);
        k_update64<ND, INTEG><<<nblk(nf, 256), 256, 0, h->stream>>>(
            h->phys, nf, (const double4_32a*)h->f_pos, (const double4_32a*)h->f_vel, h->acc, U);
        h->launches += 2;  // filter + update (the pair launch is counted by the caller)
    } else {
        Filter64 F{(float)h->grid.cs, lo2, hi2, zero2, h->f_test, h->w_test, h->l_ff, h->c_ff,
                   h->l_fw, h->c_fw, h->e_ff, h->e_fw};
        k_pair64<ND, INTEG><<<nblk(nf, h->pair_block), h->pair_block, 0, h->stream>>>(
            h->phys, nf, (const double4_32a*)h->f_pos, (const double4_32a*)h->f_vel,
            (const double4_32a*)h->f_aux, F, (const double4_32a*)h->w_pos,
            (const double4_32a*)h->w_state, U);
    }
}

void fp64_pair_kick(tp_handle* h, double* dv) {
    if (h->cfg.n_fluid == 0) return;
    Update64 U{};
    U.dv = dv;
    U.perm = h->f_perm;
    if (h->cfg.ndims == 2)
        launch_pair64<2, false>(h, U);
    else
        launch_pair64<3, false>(h, U);
}

// Stage update in place on the slot-ordered state `out` written by the pack of this stage.
void fp64_pair_stage(tp_handle* h, PhysState& out, double A, double B, double dt, int first) {
    if (h->cfg.n_fluid == 0) return;
    Update64 U{};
    U.perm = h->f_perm;
    U.u_out = out.u;
    U.v_out = (double*)out.v;
    U.tu = out.tu;
    U.tv = (double*)out.tv;
    U.xb = h->x_build;
    U.gate_next = h->gate + 3;
    U.A = A;
    U.B = B;
    U.dt = dt;
    U.first = first;
    if (h->cfg.ndims == 2)
        launch_pair64<2, true>(h, U);
    else
        launch_pair64<3, true>(h, U);
}

void fp64_count(tp_handle* h, int* nnb_ff, int* nnb_fw, int* nnb_wf) {
    const int nf = (int)h->cfg.n_fluid, nw = (int)h->cfg.n_wall;
    const double sr2 = h->phys.sr2;
    auto run = [&](auto ndc) {
        constexpr int ND = decltype(ndc)::value;
        if (nnb_ff && nf)
            k_count64<ND><<<nblk(nf, 128), 128, 0, h->stream>>>(
                h->grid, sr2, nf, (const double4_32a*)h->f_pos, h->f_skey, h->f_perm,
                (const double4_32a*)h->f_pos, h->f_start, nnb_ff);
        if (nnb_fw && nf)
            k_count64<ND><<<nblk(nf, 128), 128, 0, h->stream>>>(
                h->grid, sr2, nf, (const double4_32a*)h->f_pos, h->f_skey, h->f_perm,
                (const double4_32a*)h->w_pos, h->w_start, nnb_fw);
        if (nnb_wf && nw)
            k_count64<ND><<<nblk(nw, 128), 128, 0, h->stream>>>(
                h->grid, sr2, nw, (const double4_32a*)h->w_pos, h->w_skey, h->w_perm,
                (const double4_32a*)h->f_pos, h->f_start, nnb_wf);
    };
    if (h->cfg.ndims == 2)
        run(std::integral_constant<int, 2>{});
    else
        run(std::integral_constant<int, 3>{});
}

// The divisions of the pair kernels over caller arrays (tp_div_fast): FP64 div_fast as the
// drop-in evaluates it (x * fast_inv(y)) and the FP32 form's __fdividef.
__global__ void k_div_fast(double x64, const double* __restrict__ y64, double* __restrict__ out64,
                           float x32, const float* __restrict__ y32, float* __restrict__ out32,
                           long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (y64) out64[i] = div_fast(x64, y64[i]);
    if (y32) out32[i] = __fdividef(x32, y32[i]);
}

void div_fast_check(tp_handle* h, double x64, const double* y64, double* out64, float x32,
                    const float* y32, float* out32, long long n) {
    k_div_fast<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(x64, y64, out64, x32, y32,
                                                                     out32, n);
}

// The pair distance of the FP64 kernels over caller arrays (tp_pair_distance).
__global__ void k_pair_distance(const double* __restrict__ d2, double* __restrict__ r,
                                long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = pair_distance(d2[i]);
}

void pair_distance_check(tp_handle* h, const double* d2, double* r, long long n) {
    k_pair_distance<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(d2, r, n);
}

}  // namespace tp
