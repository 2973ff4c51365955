// tp_adjoint.cu — differentiation form: a hand-written adjoint (reverse mode) of the fused WCSPH
// right-hand side and of the CarpenterKennedy2N54 integrator (sm_103a).
//
// Forward: the same right-hand side as the integrator (rhs.jl:5-127 with the Adami gather of
// dummy_particles.jl:586-672 and gravity) in the handle's precision -- float for the FP32 form
// (pair arithmetic on FP64 position differences rounded to FP32, FP32 Kahan sums, __fdividef),
// double for the FP64 form -- with the state kept in caller order.  Neighbour lists are built at
// the start of every step at radius 2h (1 + skin) and held fixed for the step's five stages
// (pairs are still decided by |x_a - x_b|^2 <= (2h)^2 at every stage); a device check flags a
// particle that moved further than the skin allows within a step.  The state is checkpointed
// every k steps.
//
// Backward: for each k-step segment, last to first, the segment is recomputed from its
// checkpoint with every stage input recorded on a tape; then the stages are reversed:
//   U_{i+1} = U_i + B_i dU_{i+1},  dU_{i+1} = A_i dU_i + dt f(U_i)
//   =>  lam_dU += B_i lam_U;  lam_f = dt lam_dU;  lam_dU = A_i lam_dU;  lam_U += J_f(U_i)^T lam_f.
// J_f^T lam_f is hand-derived per pair: every fluid particle a recomputes its pair terms and
// pushes the reverse sweep of each term into its own adjoint (registers) and into its
// neighbour's adjoint (atomics); wall pressures and densities receive adjoints the same way and
// are then pulled back through the clipped, EOS-inverted Adami average onto the fluid.
// Parameter adjoints (Monaghan alpha, Molteni-Colagrossi delta, gravity magnitude) are reduced
// in FP64.  The WendlandC2 kernel and its gradient vanish at r = 2h, so holding the candidate
// lists fixed loses no derivative terms.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "tp_api_internal.h"
#include "tp_lists.cuh"

namespace tp {

constexpr int kAdjErrSkin = 8;  // error bit: a particle outran the list skin within a step

template <typename T>
struct AdjPhys {
    T h_inv, sr2, two_h, almostzero, wc2_norm, wc2_dnorm, hi2;
    T rho0, B, gamma, inv_gamma, p_bg, p_off;
    T beta, visc_h, visc_eps_h2, visc_ac, c, diff_coef, diff_dcoef;
    T g[3], ghat[3];
    int visc, diff, fluid_clip, wall_clip;
};

template <typename T>
struct AState {
    double* x;  // (ND, n) positions
    T* v;       // (ND, n) velocities
    T* r;       // (n) density deviation rho - rho0
};

template <typename T>
__device__ __forceinline__ T fdiv(T a, T b);
template <>
__device__ __forceinline__ float fdiv<float>(float a, float b) {
    return __fdividef(a, b);
}
template <>
__device__ __forceinline__ double fdiv<double>(double a, double b) {
    return a / b;
}

template <typename T>
struct Acc;  // per-particle sum: Kahan-compensated in float, plain in double
template <>
struct Acc<float> {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s - c; }
};
template <>
struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
};

__device__ __forceinline__ float t_expm1(float x) { return expm1f(x); }
__device__ __forceinline__ double t_expm1(double x) { return expm1(x); }
__device__ __forceinline__ float t_log1p(float x) { return log1pf(x); }
__device__ __forceinline__ double t_log1p(double x) { return log1p(x); }
__device__ __forceinline__ float t_exp(float x) { return expf(x); }
__device__ __forceinline__ double t_exp(double x) { return exp(x); }
__device__ __forceinline__ float t_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double t_sqrt(double x) { return sqrt(x); }

// Cole EOS on the density deviation and its derivative dp/d(rho - rho0).
template <typename T>
__device__ __forceinline__ T a_eos(T dr, const AdjPhys<T>& P) {
    T p = P.B * t_expm1(P.gamma * t_log1p(dr / P.rho0)) + P.p_bg;
    if (P.fluid_clip) p = (p != p || p > T(0)) ? p : T(0);
    return p;
}
template <typename T>
__device__ __forceinline__ T a_eos_deriv(T dr, const AdjPhys<T>& P) {
    const T p = P.B * t_expm1(P.gamma * t_log1p(dr / P.rho0)) + P.p_bg;
    if (P.fluid_clip && !(p > T(0))) return T(0);
    return (P.B * P.gamma / P.rho0) * t_exp((P.gamma - T(1)) * t_log1p(dr / P.rho0));
}
// Inverse EOS (density deviation of pressure p) and its derivative.
template <typename T>
__device__ __forceinline__ T a_eos_inv(T p, const AdjPhys<T>& P) {
    return P.rho0 * t_expm1(t_log1p((p - P.p_bg) / P.B) * P.inv_gamma);
}
template <typename T>
__device__ __forceinline__ T a_eos_inv_deriv(T p, const AdjPhys<T>& P) {
    return (P.rho0 / (P.B * P.gamma)) * t_exp((P.inv_gamma - T(1)) * t_log1p((p - P.p_bg) / P.B));
}

template <typename T, int ND>
__device__ __forceinline__ T pos_diff(const double* __restrict__ xa, const double* __restrict__ xb,
                                      T pd[3]) {
    T d2 = T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        pd[d] = (d < ND) ? (T)(xa[d] - xb[d]) : T(0);
        d2 += pd[d] * pd[d];
    }
    return d2;
}

// The per-particle kernels of the adjoint run kAdjLanes threads per particle (or wall particle),
// each over every kAdjLanes-th entry of its lists: the differentiated problems are small (tens of
// thousands of particles), and one thread per particle leaves a few warps per SM walking their
// lists one dependent load at a time.  Lane partial sums are combined with shuffles inside the
// group of kAdjLanes consecutive lanes.
constexpr int kAdjLanes = 4;

template <typename T>
__device__ __forceinline__ T lane_group_sum(T x) {
#pragma unroll
    for (int off = kAdjLanes / 2; off > 0; off >>= 1)
        x += __shfl_down_sync(0xffffffffu, x, off, kAdjLanes);
    return x;  // complete in the group's first lane
}

// ------------------------------------------------------------------------------------------
// Neighbour lists in caller order (entry k of particle i at list[k * n + i]).  The search covers
// the +-1 cells and reaches a second cell along an axis where the point lies within
// m = r_list - cs of that cell face (the list radius exceeds the 2h cell size).
// ------------------------------------------------------------------------------------------
struct CellReach {
    int lo[3], hi[3];  // inclusive cell ranges, clamped to the grid
};

__device__ __forceinline__ CellReach cell_reach(const GridDesc& g, const int c[3],
                                                const double* x, int nd, double m) {
    CellReach R;
    for (int d = 0; d < 3; ++d) {
        if (d < nd) {
            const double o = x[d] - (double)(g.cmin[d] + c[d]) * g.cs;
            R.lo[d] = max(c[d] - (o <= m ? 2 : 1), 0);
            R.hi[d] = min(c[d] + (o >= g.cs - m ? 2 : 1), g.n[d] - 1);
        } else {
            R.lo[d] = R.hi[d] = 0;
        }
    }
    return R;
}

template <int ND>
__global__ void __launch_bounds__(128) k_adj_fluid_lists(
    GridDesc g, double rl2, double m, int nf, const double* __restrict__ x,
    const int* __restrict__ key, const int* __restrict__ fstart, const int* __restrict__ fperm,
    const double4_32a* __restrict__ wpos, const int* __restrict__ wstart, int* __restrict__ ff,
    int* __restrict__ ffc, int cap_ff, int* __restrict__ fw, int* __restrict__ fwc, int cap_fw,
    double* __restrict__ xb, int* __restrict__ err) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nf) return;
    double xa[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        xa[d] = x[(size_t)a * ND + d];
        xb[(size_t)a * ND + d] = xa[d];
    }
    int c[3];
    key_to_coords(key[a], g, c);
    const CellReach R = cell_reach(g, c, xa, ND, m);
    int n1 = 0, n2 = 0;
    for (int cz = R.lo[2]; cz <= R.hi[2]; ++cz)
        for (int cy = R.lo[1]; cy <= R.hi[1]; ++cy) {
            const int rb = g.n[0] * (cy + g.n[1] * cz);
            for (int s = fstart[rb + R.lo[0]]; s < fstart[rb + R.hi[0] + 1]; ++s) {
                const int b = fperm[s];
                if (b == a) continue;
                double d2 = 0.0;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const double e = xa[d] - x[(size_t)b * ND + d];
                    d2 += e * e;
                }
                if (d2 <= rl2) {
                    if (n1 < cap_ff) ff[(size_t)n1 * nf + a] = b;
                    ++n1;
                }
            }
            for (int w = wstart[rb + R.lo[0]]; w < wstart[rb + R.hi[0] + 1]; ++w) {
                const double4_32a pw = wpos[w];
                const double pwx[3] = {pw.x, pw.y, pw.z};
                double d2 = 0.0;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const double e = xa[d] - pwx[d];
                    d2 += e * e;
                }
                if (d2 <= rl2) {
                    if (n2 < cap_fw) fw[(size_t)n2 * nf + a] = w;
                    ++n2;
                }
            }
        }
    ffc[a] = min(n1, cap_ff);
    fwc[a] = min(n2, cap_fw);
    if (n1 > cap_ff || n2 > cap_fw) atomicOr(err, TP_ERRBIT_CAPACITY);
}

template <int ND>
__global__ void __launch_bounds__(128) k_adj_wall_lists(
    GridDesc g, double rl2, double m, int nw, const double4_32a* __restrict__ wpos,
    const int* __restrict__ wskey, const double* __restrict__ x, const int* __restrict__ fstart,
    const int* __restrict__ fperm, int* __restrict__ wf, int* __restrict__ wfc, int cap_wf,
    int* __restrict__ err) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    const double4_32a pw = wpos[w];
    const double xw[3] = {pw.x, pw.y, pw.z};
    int c[3];
    key_to_coords(wskey[w], g, c);
    const CellReach R = cell_reach(g, c, xw, ND, m);
    int n1 = 0;
    for (int cz = R.lo[2]; cz <= R.hi[2]; ++cz)
        for (int cy = R.lo[1]; cy <= R.hi[1]; ++cy) {
            const int rb = g.n[0] * (cy + g.n[1] * cz);
            for (int s = fstart[rb + R.lo[0]]; s < fstart[rb + R.hi[0] + 1]; ++s) {
                const int b = fperm[s];
                double d2 = 0.0;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const double e = xw[d] - x[(size_t)b * ND + d];
                    d2 += e * e;
                }
                if (d2 <= rl2) {
                    if (n1 < cap_wf) wf[(size_t)n1 * nw + w] = b;
                    ++n1;
                }
            }
        }
    wfc[w] = min(n1, cap_wf);
    if (n1 > cap_wf) atomicOr(err, TP_ERRBIT_CAPACITY);
}

// Largest displacement since the list build above skin * h -> error bit.
template <int ND>
__global__ void k_adj_skin_check(const double* __restrict__ x, const double* __restrict__ xb,
                                 int n, double lim2, int* __restrict__ err) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    double d2 = 0.0;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const double e = x[(size_t)a * ND + d] - xb[(size_t)a * ND + d];
        d2 += e * e;
    }
    if (!(d2 <= lim2)) atomicOr(err, kAdjErrSkin);
}

// ------------------------------------------------------------------------------------------
// State load / store (reference layout v = (ND+1, n) with density last, u = (ND, n))
// ------------------------------------------------------------------------------------------
template <typename T, int ND>
__global__ void k_adj_load(const double* __restrict__ v, const double* __restrict__ u,
                           const double* __restrict__ m, double rho0, AState<T> s,
                           T* __restrict__ mt, int n) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        s.x[(size_t)a * ND + d] = u[(size_t)a * ND + d];
        s.v[(size_t)a * ND + d] = (T)v[(size_t)a * (ND + 1) + d];
    }
    s.r[a] = (T)(v[(size_t)a * (ND + 1) + ND] - rho0);
    mt[a] = (T)m[a];
}

template <typename T, int ND>
__global__ void k_adj_store(AState<T> s, double rho0, double* __restrict__ v,
                            double* __restrict__ u, int n) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        u[(size_t)a * ND + d] = s.x[(size_t)a * ND + d];
        v[(size_t)a * (ND + 1) + d] = (double)s.v[(size_t)a * ND + d];
    }
    v[(size_t)a * (ND + 1) + ND] = (double)s.r[a] + rho0;
}

template <typename T, int ND>
__global__ void k_adj_copy(AState<T> src, AState<T> dst, int n) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        dst.x[(size_t)a * ND + d] = src.x[(size_t)a * ND + d];
        dst.v[(size_t)a * ND + d] = src.v[(size_t)a * ND + d];
    }
    dst.r[a] = src.r[a];
}

// Fluid pressures of a state (one EOS per particle per stage).
template <typename T>
__global__ void k_adj_pressure(AdjPhys<T> P, const T* __restrict__ r, T* __restrict__ p, int n) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) p[a] = a_eos(r[a], P);
}

// ------------------------------------------------------------------------------------------
// Forward: Adami wall state and the fused stage (pair sums + 2N update)
// ------------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T wc2_kernel(T r, const AdjPhys<T>& P) {
    if (!(r < P.two_h)) return T(0);
    const T q = r * P.h_inv;
    const T t = T(1) - T(0.5) * q;
    const T t2 = t * t;
    return (P.wc2_norm * (t2 * t2)) * (T(2) * q + T(1));
}

template <typename T, int ND>
__global__ void __launch_bounds__(128) k_adj_adami(AdjPhys<T> P, int nw,
                                                   const double4_32a* __restrict__ wpos,
                                                   const int* __restrict__ wf,
                                                   const int* __restrict__ wfc, AState<T> s,
                                                   const T* __restrict__ pf, T* __restrict__ wp,
                                                   T* __restrict__ wr, T* __restrict__ wnum,
                                                   T* __restrict__ wvol) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = gt / kAdjLanes, sub = gt % kAdjLanes;
    const bool active = w < nw;
    const double4_32a pw = wpos[active ? w : 0];
    const double xw[3] = {pw.x, pw.y, pw.z};
    Acc<T> Ps, V;
    const int n = active ? wfc[w] : 0;
    for (int k = sub; k < n; k += kAdjLanes) {
        const int f = wf[(size_t)k * nw + w];
        T pd[3];
        const T d2 = pos_diff<T, ND>(xw, s.x + (size_t)f * ND, pd);
        if (d2 > P.sr2) continue;
        const T r = t_sqrt(d2);
        const T rho_f = P.rho0 + s.r[f];
        T hp = T(0);
#pragma unroll
        for (int d = 0; d < ND; ++d) hp += P.g[d] * (rho_f * pd[d]);
        const T sum = (P.p_off + pf[f]) + hp;
        const T W = wc2_kernel(r, P);
        Ps.add(sum * W);
        V.add(W);
    }
    const T num = lane_group_sum(Ps.value()), vol = lane_group_sum(V.value());
    if (!active || sub != 0) return;
    T p = num;
    if ((double)vol > 2.220446049250313e-16) p = p / vol;
    if (P.wall_clip) p = (p != p || p > T(0)) ? p : T(0);
    wp[w] = p;
    wr[w] = a_eos_inv(p, P);
    wnum[w] = num;
    wvol[w] = vol;
}

template <typename T>
struct AdjStage {
    T A, B, dt;
    double Ad, Bd, dtd;
    int first;
};

template <typename T, int ND>
__global__ void __launch_bounds__(128) k_adj_stage(
    AdjPhys<T> P, int nf, AState<T> src, AState<T> dst, const T* __restrict__ pf,
    const T* __restrict__ mf, const int* __restrict__ ff, const int* __restrict__ ffc,
    const int* __restrict__ fw, const int* __restrict__ fwc, const double4_32a* __restrict__ wpos,
    const T* __restrict__ wp, const T* __restrict__ wr, double* __restrict__ tx,
    T* __restrict__ tv, T* __restrict__ tr, AdjStage<T> S) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int sub = gt % kAdjLanes;
    const bool active = gt / kAdjLanes < nf;
    const int a = active ? gt / kAdjLanes : 0;
    const double* xa = src.x + (size_t)a * ND;
    T va[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int d = 0; d < ND; ++d) va[d] = src.v[(size_t)a * ND + d];
    const T ra = src.r[a], p_a = pf[a], rho_a = P.rho0 + ra;

    Acc<T> dv[3], dr;
    const int nff = active ? ffc[a] : 0;
    for (int k = sub; k < nff; k += kAdjLanes) {
        const int b = ff[(size_t)k * nf + a];
        T pd[3];
        const T d2 = pos_diff<T, ND>(xa, src.x + (size_t)b * ND, pd);
        if (d2 > P.sr2) continue;
        const T r = t_sqrt(d2);
        if (r < P.almostzero) continue;
        T vb[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int d = 0; d < ND; ++d) vb[d] = src.v[(size_t)b * ND + d];
        const T rb = src.r[b], m_b = mf[b], p_b = pf[b], rho_b = P.rho0 + rb;
        const T q = r * P.h_inv;
        const T t = T(1) - T(0.5) * q;
        const T sg = (P.wc2_dnorm * ((t * t) * t)) * P.hi2;
        T gk[3], vd[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            gk[d] = sg * pd[d];
            vd[d] = va[d] - vb[d];
        }
        const T coef = -m_b * fdiv(p_a + p_b, rho_a * rho_b);
        T e[3] = {coef * gk[0], coef * gk[1], coef * gk[2]};
        if (P.visc) {
            T vr = T(0);
#pragma unroll
            for (int d = 0; d < ND; ++d) vr += vd[d] * pd[d];
            if (vr < T(0)) {
                const T rho_mean = T(0.5) * (rho_a + rho_b);
                const T mu = fdiv(P.visc_h * vr, r * r + P.visc_eps_h2);
                const T num = (m_b * P.visc_ac) * mu + (m_b * P.beta) * (mu * mu);
                const T f = fdiv(num, rho_mean);
#pragma unroll
                for (int d = 0; d < 3; ++d) e[d] += f * gk[d];
            }
        }
#pragma unroll
        for (int d = 0; d < ND; ++d) dv[d].add(e[d]);
        T vg = T(0);
#pragma unroll
        for (int d = 0; d < ND; ++d) vg += vd[d] * gk[d];
        T er = (fdiv(rho_a, rho_b) * m_b) * vg;
        if (P.diff) {
            const T vol_b = fdiv(m_b, rho_b);
            const T pc = fdiv(T(2) * (ra - rb), r * r);
            T pg = T(0);
#pragma unroll
            for (int d = 0; d < ND; ++d) pg += pd[d] * gk[d];
            er += P.diff_coef * (vol_b * (pc * pg));
        }
        dr.add(er);
    }
    const int nfw = active ? fwc[a] : 0;
    for (int k = sub; k < nfw; k += kAdjLanes) {
        const int w = fw[(size_t)k * nf + a];
        const double4_32a pw = wpos[w];
        const double xw[3] = {pw.x, pw.y, pw.z};
        T pd[3];
        const T d2 = pos_diff<T, ND>(xa, xw, pd);
        if (d2 > P.sr2) continue;
        const T r = t_sqrt(d2);
        if (r < P.almostzero) continue;
        const T m_w = (T)pw.w, p_w = wp[w], rho_w = P.rho0 + wr[w];
        const T q = r * P.h_inv;
        const T t = T(1) - T(0.5) * q;
        const T sg = (P.wc2_dnorm * ((t * t) * t)) * P.hi2;
        const T coef = -m_w * fdiv(p_a + p_w, rho_a * rho_w);
        T vg = T(0);
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            dv[d].add(coef * (sg * pd[d]));
            vg += va[d] * (sg * pd[d]);
        }
        dr.add((fdiv(rho_a, rho_w) * m_w) * vg);
    }
    T dvs[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int d = 0; d < ND; ++d) dvs[d] = lane_group_sum(dv[d].value());
    const T drs = lane_group_sum(dr.value());
    if (!active || sub != 0) return;

    // CarpenterKennedy2N54 stage on (x, v, rho - rho0): t = A t + dt k ; y = y + B t
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const T kv = dvs[d] + P.g[d];
        const T tvd = S.first ? S.dt * kv : S.dt * kv + S.A * tv[(size_t)a * ND + d];
        tv[(size_t)a * ND + d] = tvd;
        dst.v[(size_t)a * ND + d] = va[d] + S.B * tvd;
        const double ku = (double)va[d];
        const double txd = S.first ? S.dtd * ku : fma(S.dtd, ku, S.Ad * tx[(size_t)a * ND + d]);
        tx[(size_t)a * ND + d] = txd;
        dst.x[(size_t)a * ND + d] = fma(S.Bd, txd, xa[d]);
    }
    const T kr = drs;
    const T trd = S.first ? S.dt * kr : S.dt * kr + S.A * tr[a];
    tr[a] = trd;
    dst.r[a] = ra + S.B * trd;
}

// ------------------------------------------------------------------------------------------
// Backward
// ------------------------------------------------------------------------------------------
template <typename T>
struct AdjLam {
    T* x;    // (ND, n) adjoint of positions
    T* v;    // (ND, n) adjoint of velocities
    T* r;    // (n)     adjoint of the density deviation
    T* p;    // (n)     adjoint of fluid pressures (pulled back through the EOS per stage)
    T* dx;   // adjoints of the 2N registers
    T* dv;
    T* dr;
    T* fv;   // (ND, n) adjoint of the stage's dv output (= dt lam_dU)
    T* fr;   // (n)     adjoint of the stage's drho output
    T* wp;   // (nw)    adjoint of wall pressures
    T* wr;   // (nw)    adjoint of wall density deviations
};

// lam_dU += B lam_U ; lam_f = dt lam_dU ; lam_dU = A lam_dU ; lam_v += lam_f(x part)
template <typename T, int ND>
__global__ void k_adj_seed(AdjLam<T> L, T A, T B, T dt, int n, int nw) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < nw) {
        L.wp[a] = T(0);
        L.wr[a] = T(0);
    }
    if (a >= n) return;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const size_t i = (size_t)a * ND + d;
        T ldx = L.dx[i] + B * L.x[i];
        const T fx = dt * ldx;
        L.dx[i] = A * ldx;
        T ldv = L.dv[i] + B * L.v[i];
        L.fv[i] = dt * ldv;
        L.dv[i] = A * ldv;
        L.v[i] += fx;  // du = v
    }
    T ldr = L.dr[a] + B * L.r[a];
    L.fr[a] = dt * ldr;
    L.dr[a] = A * ldr;
}

__device__ __forceinline__ void atomic_add_t(float* p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_t(double* p, double v) { atomicAdd(p, v); }

// Block sum of three doubles into theta[0..2] (FP64 gradient reduction).
__device__ __forceinline__ void reduce_theta(double a, double b, double c,
                                             double* __restrict__ theta) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
        c += __shfl_xor_sync(0xffffffffu, c, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (a != 0.0) atomicAdd(&theta[0], a);
        if (b != 0.0) atomicAdd(&theta[1], b);
        if (c != 0.0) atomicAdd(&theta[2], c);
    }
}

// Reverse sweep of the fluid pair terms of particle a (fluid-fluid and fluid-wall) and of
// gravity, seeded with lam_f(a).  theta = (alpha, delta, gravity magnitude).
template <typename T, int ND>
__global__ void __launch_bounds__(128) k_adj_pair_vjp(
    AdjPhys<T> P, int nf, AState<T> s, const T* __restrict__ pf, const T* __restrict__ mf,
    const int* __restrict__ ff, const int* __restrict__ ffc, const int* __restrict__ fw,
    const int* __restrict__ fwc, const double4_32a* __restrict__ wpos, const T* __restrict__ wp,
    const T* __restrict__ wr, AdjLam<T> L, double* __restrict__ theta) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = gt / kAdjLanes, sub = gt % kAdjLanes;
    double th_alpha = 0.0, th_delta = 0.0, th_g = 0.0;
    if (a < nf) {
        const double* xa = s.x + (size_t)a * ND;
        T va[3] = {T(0), T(0), T(0)}, Lv[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            va[d] = s.v[(size_t)a * ND + d];
            Lv[d] = L.fv[(size_t)a * ND + d];
        }
        const T Lr = L.fr[a];
        const T ra = s.r[a], p_a = pf[a], rho_a = P.rho0 + ra;
        T xa_bar[3] = {T(0), T(0), T(0)}, va_bar[3] = {T(0), T(0), T(0)};
        T ra_bar = T(0), pa_bar = T(0);
        // gravity: dv_a += |g| ghat (once per particle)
        if (sub == 0) {
#pragma unroll
            for (int d = 0; d < ND; ++d) th_g += (double)Lv[d] * (double)P.ghat[d];
        }

        const int nff = ffc[a];
        for (int k = sub; k < nff; k += kAdjLanes) {
            const int b = ff[(size_t)k * nf + a];
            T pd[3];
            const T d2 = pos_diff<T, ND>(xa, s.x + (size_t)b * ND, pd);
            if (d2 > P.sr2) continue;
            const T r = t_sqrt(d2);
            if (r < P.almostzero) continue;
            T vb[3] = {T(0), T(0), T(0)};
#pragma unroll
            for (int d = 0; d < ND; ++d) vb[d] = s.v[(size_t)b * ND + d];
            const T rb = s.r[b], m_b = mf[b], p_b = pf[b], rho_b = P.rho0 + rb;
            // forward recompute
            const T q = r * P.h_inv;
            const T t = T(1) - T(0.5) * q;
            const T sg = (P.wc2_dnorm * ((t * t) * t)) * P.hi2;
            T gk[3], vd[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                gk[d] = sg * pd[d];
                vd[d] = va[d] - vb[d];
            }
            const T Pab = p_a + p_b, Q = rho_a * rho_b;
            const T coef = -m_b * (Pab / Q);
            T vr = T(0), vg = T(0), pg = T(0), Lg = T(0);
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                vr += vd[d] * pd[d];
                vg += vd[d] * gk[d];
                pg += pd[d] * gk[d];
                Lg += Lv[d] * gk[d];
            }
            const bool visc_on = P.visc && vr < T(0);
            T rho_mean = T(0), den = T(1), mu = T(0), f = T(0);
            if (visc_on) {
                rho_mean = T(0.5) * (rho_a + rho_b);
                den = r * r + P.visc_eps_h2;
                mu = P.visc_h * vr / den;
                const T num = (m_b * P.visc_ac) * mu + (m_b * P.beta) * (mu * mu);
                f = num / rho_mean;
            }
            const T Kc = (rho_a / rho_b) * m_b;
            // reverse
            T gbar[3] = {T(0), T(0), T(0)}, pdbar[3] = {T(0), T(0), T(0)};
            T vdbar[3] = {T(0), T(0), T(0)};
            T rbar = T(0), rho_a_bar = T(0), rho_b_bar = T(0);
            // er1 = Kc * vg
            const T vgbar = Lr * Kc;
            rho_a_bar += Lr * m_b * vg / rho_b;
            rho_b_bar -= Lr * Kc * vg / rho_b;
            if (P.diff) {
                const T vol_b = m_b / rho_b;
                const T rr = r * r;
                const T pc = T(2) * (ra - rb) / rr;
                const T sd = Lr * P.diff_coef;
                th_delta += (double)Lr * (double)P.diff_dcoef * (double)(vol_b * (pc * pg));
                const T volb_bar = sd * pc * pg;
                rho_b_bar -= volb_bar * vol_b / rho_b;
                const T pc_bar = sd * vol_b * pg;
                rho_a_bar += pc_bar * T(2) / rr;
                rho_b_bar -= pc_bar * T(2) / rr;
                rbar -= pc_bar * T(2) * pc / r;
                const T pg_bar = sd * vol_b * pc;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    pdbar[d] += pg_bar * gk[d];
                    gbar[d] += pg_bar * pd[d];
                }
            }
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                vdbar[d] += vgbar * gk[d];
                gbar[d] += vgbar * vd[d] + (coef + f) * Lv[d];
            }
            const T coef_bar = Lg;
            if (visc_on) {
                const T f_bar = Lg;
                const T num_bar = f_bar / rho_mean;
                const T rhom_bar = -f_bar * f / rho_mean;
                rho_a_bar += T(0.5) * rhom_bar;
                rho_b_bar += T(0.5) * rhom_bar;
                const T mu_bar = num_bar * (m_b * P.visc_ac + T(2) * m_b * P.beta * mu);
                th_alpha += (double)num_bar * (double)(m_b * P.c) * (double)mu;
                const T vr_bar = mu_bar * P.visc_h / den;
                const T den_bar = -mu_bar * mu / den;
                rbar += den_bar * T(2) * r;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    vdbar[d] += vr_bar * pd[d];
                    pdbar[d] += vr_bar * vd[d];
                }
            }
            const T pab_bar = coef_bar * (-m_b / Q);
            pa_bar += pab_bar;
            const T Q_bar = -coef_bar * coef / Q;
            rho_a_bar += Q_bar * rho_b;
            rho_b_bar += Q_bar * rho_a;
            T sg_bar = T(0);
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                sg_bar += gbar[d] * pd[d];
                pdbar[d] += sg * gbar[d];
            }
            const T t_bar = sg_bar * P.wc2_dnorm * P.hi2 * T(3) * t * t;
            rbar += T(-0.5) * t_bar * P.h_inv;
            const T rs = rbar / r;
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                pdbar[d] += rs * pd[d];
                xa_bar[d] += pdbar[d];
                va_bar[d] += vdbar[d];
                atomic_add_t(&L.x[(size_t)b * ND + d], -pdbar[d]);
                atomic_add_t(&L.v[(size_t)b * ND + d], -vdbar[d]);
            }
            ra_bar += rho_a_bar;
            atomic_add_t(&L.r[b], rho_b_bar);
            atomic_add_t(&L.p[b], pab_bar);
        }

        const int nfw = fwc[a];
        for (int k = sub; k < nfw; k += kAdjLanes) {
            const int w = fw[(size_t)k * nf + a];
            const double4_32a pw = wpos[w];
            const double xw[3] = {pw.x, pw.y, pw.z};
            T pd[3];
            const T d2 = pos_diff<T, ND>(xa, xw, pd);
            if (d2 > P.sr2) continue;
            const T r = t_sqrt(d2);
            if (r < P.almostzero) continue;
            const T m_w = (T)pw.w, p_w = wp[w], rho_w = P.rho0 + wr[w];
            const T q = r * P.h_inv;
            const T t = T(1) - T(0.5) * q;
            const T sg = (P.wc2_dnorm * ((t * t) * t)) * P.hi2;
            const T Q = rho_a * rho_w;
            const T coef = -m_w * ((p_a + p_w) / Q);
            T gk[3], vg = T(0), Lg = T(0);
#pragma unroll
            for (int d = 0; d < 3; ++d) gk[d] = sg * pd[d];
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                vg += va[d] * gk[d];
                Lg += Lv[d] * gk[d];
            }
            const T Kc = (rho_a / rho_w) * m_w;
            const T vgbar = Lr * Kc;
            T rho_a_bar = Lr * m_w * vg / rho_w;
            T rho_w_bar = -Lr * Kc * vg / rho_w;
            T gbar[3];
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                va_bar[d] += vgbar * gk[d];
                gbar[d] = vgbar * va[d] + coef * Lv[d];
            }
            const T pab_bar = Lg * (-m_w / Q);
            pa_bar += pab_bar;
            const T Q_bar = -Lg * coef / Q;
            rho_a_bar += Q_bar * rho_w;
            rho_w_bar += Q_bar * rho_a;
            T sg_bar = T(0);
#pragma unroll
            for (int d = 0; d < ND; ++d) sg_bar += gbar[d] * pd[d];
            const T t_bar = sg_bar * P.wc2_dnorm * P.hi2 * T(3) * t * t;
            const T rs = (T(-0.5) * t_bar * P.h_inv) / r;
#pragma unroll
            for (int d = 0; d < ND; ++d) xa_bar[d] += sg * gbar[d] + rs * pd[d];
            ra_bar += rho_a_bar;
            atomic_add_t(&L.wp[w], pab_bar);
            atomic_add_t(&L.wr[w], rho_w_bar);
        }
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            atomic_add_t(&L.x[(size_t)a * ND + d], xa_bar[d]);
            atomic_add_t(&L.v[(size_t)a * ND + d], va_bar[d]);
        }
        atomic_add_t(&L.r[a], ra_bar);
        atomic_add_t(&L.p[a], pa_bar);
    }
    reduce_theta(th_alpha, th_delta, th_g, theta);
}

// Reverse sweep of the Adami wall state of wall w onto the fluid.
template <typename T, int ND>
__global__ void __launch_bounds__(128) k_adj_adami_vjp(
    AdjPhys<T> P, int nw, const double4_32a* __restrict__ wpos, const int* __restrict__ wf,
    const int* __restrict__ wfc, AState<T> s, const T* __restrict__ pf,
    const T* __restrict__ wp, const T* __restrict__ wnum, const T* __restrict__ wvol,
    AdjLam<T> L, double* __restrict__ theta) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = gt / kAdjLanes, sub = gt % kAdjLanes;
    double th_g = 0.0;
    if (w < nw) {
        const T p = wp[w], num = wnum[w], vol = wvol[w];
        const bool divided = (double)vol > 2.220446049250313e-16;
        const T p_pre = divided ? num / vol : num;
        const bool clipped = P.wall_clip && !(p_pre != p_pre || p_pre > T(0));
        const T pbar = L.wp[w] + L.wr[w] * a_eos_inv_deriv(p, P);
        const T pre_bar = clipped ? T(0) : pbar;
        const T N_bar = divided ? pre_bar / vol : pre_bar;
        const T V_bar = divided ? -pre_bar * p_pre / vol : T(0);
        if (N_bar != T(0) || V_bar != T(0)) {
            const double4_32a pw = wpos[w];
            const double xw[3] = {pw.x, pw.y, pw.z};
            const int n = wfc[w];
            for (int k = sub; k < n; k += kAdjLanes) {
                const int f = wf[(size_t)k * nw + w];
                T pd[3];
                const T d2 = pos_diff<T, ND>(xw, s.x + (size_t)f * ND, pd);
                if (d2 > P.sr2) continue;
                const T r = t_sqrt(d2);
                const T rho_f = P.rho0 + s.r[f];
                T hp = T(0), gp = T(0), ghp = T(0);
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    hp += P.g[d] * (rho_f * pd[d]);
                    gp += P.g[d] * pd[d];
                    ghp += P.ghat[d] * pd[d];
                }
                const T sum = (P.p_off + pf[f]) + hp;
                const T W = wc2_kernel(r, P);
                const T sum_bar = N_bar * W;
                const T W_bar = N_bar * sum + V_bar;
                th_g += (double)sum_bar * (double)rho_f * (double)ghp;
                T pdbar[3];
#pragma unroll
                for (int d = 0; d < ND; ++d) pdbar[d] = sum_bar * rho_f * P.g[d];
                if (r < P.two_h && r > T(0)) {
                    const T q = r * P.h_inv;
                    const T t = T(1) - T(0.5) * q;
                    const T dWdr = T(-5) * P.wc2_norm * q * (t * t * t) * P.h_inv;
                    const T rs = W_bar * dWdr / r;
#pragma unroll
                    for (int d = 0; d < ND; ++d) pdbar[d] += rs * pd[d];
                }
#pragma unroll
                for (int d = 0; d < ND; ++d) atomic_add_t(&L.x[(size_t)f * ND + d], -pdbar[d]);
                atomic_add_t(&L.p[f], sum_bar);
                atomic_add_t(&L.r[f], sum_bar * gp);
            }
        }
    }
    reduce_theta(0.0, 0.0, th_g, theta);
}

// lam_r += lam_p * dp/drho ; lam_p = 0
template <typename T>
__global__ void k_adj_eos_vjp(AdjPhys<T> P, const T* __restrict__ r, AdjLam<T> L, int n) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const T lp = L.p[a];
    if (lp != T(0)) L.r[a] += lp * a_eos_deriv(r[a], P);
    L.p[a] = T(0);
}

template <typename T, int ND>
__global__ void k_adj_lam_load(const double* __restrict__ vbar, const double* __restrict__ ubar,
                               AdjLam<T> L, int n) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const size_t i = (size_t)a * ND + d;
        L.x[i] = (T)ubar[i];
        L.v[i] = (T)vbar[(size_t)a * (ND + 1) + d];
        L.dx[i] = T(0);
        L.dv[i] = T(0);
    }
    L.r[a] = (T)vbar[(size_t)a * (ND + 1) + ND];
    L.dr[a] = T(0);
    L.p[a] = T(0);
}

template <typename T, int ND>
__global__ void k_adj_lam_store(AdjLam<T> L, double* __restrict__ vbar, double* __restrict__ ubar,
                                int n) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const size_t i = (size_t)a * ND + d;
        ubar[i] = (double)L.x[i];
        vbar[(size_t)a * (ND + 1) + d] = (double)L.v[i];
    }
    vbar[(size_t)a * (ND + 1) + ND] = (double)L.r[a];
}

// ------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------
struct AdjointState {
    bool f32 = false;
    int nd = 2, nf = 0, nw = 0;
    double skin = 0.1;
    // lists (caller order)
    int *ff = nullptr, *fw = nullptr, *wf = nullptr, *ffc = nullptr, *fwc = nullptr, *wfc = nullptr;
    int cap_ff = 0, cap_fw = 0, cap_wf = 0;
    double* xb = nullptr;
    // fluid masses / pressures, wall state (element type = T)
    void *mf = nullptr, *pf = nullptr, *wp = nullptr, *wr = nullptr, *wnum = nullptr,
         *wvol = nullptr;
    // 2N registers (x FP64, v and r in T)
    double* tx = nullptr;
    void *tv = nullptr, *tr = nullptr;
    // state storage: two ping-pong states, checkpoints, tape (each n * (8 ND + sT (ND + 1)))
    std::vector<void*> blocks;
    void* pingpong = nullptr;
    void* ckpt = nullptr;
    void* tape = nullptr;
    size_t n_ckpt = 0, n_tape = 0;
    // adjoints
    void* lam = nullptr;  // all adjoint arrays in one allocation
    double* theta = nullptr;
    double* h_theta = nullptr;  // pinned
    // per-segment storage of the backward pass (null when it would not fit): the neighbour lists
    // of every step and the pressure / wall state of every stage of the segment being reversed,
    // kept from its recomputation so that the reverse sweep does not rebuild them
    void* seg = nullptr;
    size_t seg_bytes = 0;
    // recorded forward
    bool recorded = false;
    double dt = 0.0;
    long long n_steps = 0, every = 0;
    long long kernels = 0;
};

namespace {

inline int nb(long n, int t) { return (int)((n + t - 1) / t); }

#define ADJ_CUDA(h, call)                                        \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return api_cuda_fail(h, e_, #call); \
    } while (0)
#define ADJ_LAUNCHED(h, where)                                   \
    do {                                                         \
        cudaError_t e_ = cudaGetLastError();                     \
        if (e_ != cudaSuccess) return api_cuda_fail(h, e_, where); \
    } while (0)

template <typename T>
size_t state_bytes(const AdjointState& A) {
    return (size_t)A.nf * (8 * A.nd + sizeof(T) * (A.nd + 1));
}

template <typename T>
AState<T> state_at(const AdjointState& A, void* base, size_t k) {
    char* p = (char*)base + k * state_bytes<T>(A);
    AState<T> s;
    s.x = (double*)p;
    s.v = (T*)(p + (size_t)A.nf * 8 * A.nd);
    s.r = (T*)(p + (size_t)A.nf * (8 * A.nd + sizeof(T) * A.nd));
    return s;
}

template <typename T>
AdjPhys<T> make_phys(const tp_handle* h) {
    const Phys& Q = h->phys;
    AdjPhys<T> P{};
    P.h_inv = (T)Q.h_inv;
    P.sr2 = (T)Q.sr2;
    P.two_h = (T)Q.two_h;
    P.almostzero = (T)Q.almostzero;
    P.wc2_norm = (T)Q.wc2_norm;
    P.wc2_dnorm = (T)Q.wc2_dnorm;
    P.hi2 = (T)Q.hi2;
    P.rho0 = (T)Q.rho0;
    P.B = (T)Q.B;
    P.gamma = (T)Q.gamma;
    P.inv_gamma = (T)Q.inv_gamma;
    P.p_bg = (T)Q.p_bg;
    P.p_off = (T)Q.p_off;
    P.beta = (T)Q.beta;
    P.visc_h = (T)Q.visc_h;
    P.visc_eps_h2 = (T)Q.visc_eps_h2;
    P.visc_ac = (T)(Q.alpha * Q.c);
    P.c = (T)Q.c;
    P.diff_coef = (T)Q.diff_coef;
    P.diff_dcoef = (T)(((Q.h + Q.h) / 2.0) * Q.c);  // d diff_coef / d delta
    double gn = 0.0;
    for (int d = 0; d < 3; ++d) gn += Q.g[d] * Q.g[d];
    gn = std::sqrt(gn);
    for (int d = 0; d < 3; ++d) {
        P.g[d] = (T)Q.g[d];
        P.ghat[d] = (T)(gn > 0.0 ? Q.g[d] / gn : 0.0);
    }
    P.visc = Q.visc;
    P.diff = Q.diff;
    P.fluid_clip = Q.fluid_clip;
    P.wall_clip = Q.wall_clip;
    return P;
}

// The neighbour lists of one step and the pressure / wall state of one stage.
struct ListSet {
    int *ff, *fw, *wf, *ffc, *fwc, *wfc;
};
template <typename T>
struct WallSet {
    T *pf, *wp, *wr, *wnum, *wvol;
};

ListSet lists_of(const AdjointState& A) {
    return ListSet{A.ff, A.fw, A.wf, A.ffc, A.fwc, A.wfc};
}
template <typename T>
WallSet<T> walls_of(const AdjointState& A) {
    return WallSet<T>{(T*)A.pf, (T*)A.wp, (T*)A.wr, (T*)A.wnum, (T*)A.wvol};
}

// Segment storage layout: `steps` list sets, then 5 * steps wall sets.
size_t list_set_ints(const AdjointState& A) {
    const size_t n = (size_t)A.nf, nw = (size_t)std::max(A.nw, 1);
    return (size_t)A.cap_ff * n + (size_t)A.cap_fw * n + (size_t)A.cap_wf * nw + 2 * n + nw;
}
template <typename T>
size_t wall_set_elems(const AdjointState& A) {
    return (size_t)A.nf + 4 * (size_t)std::max(A.nw, 1);
}
template <typename T>
size_t seg_bytes_for(const AdjointState& A, long long steps) {
    const size_t lists = ((list_set_ints(A) * 4 + 255) / 256) * 256;
    const size_t walls = ((wall_set_elems<T>(A) * sizeof(T) + 255) / 256) * 256;
    return (size_t)steps * (lists + 5 * walls);
}
ListSet seg_lists(const AdjointState& A, long long j) {
    const size_t n = (size_t)A.nf, nw = (size_t)std::max(A.nw, 1);
    const size_t lists = ((list_set_ints(A) * 4 + 255) / 256) * 256;
    int* p = (int*)((char*)A.seg + (size_t)j * lists);
    ListSet L;
    L.ff = p;
    p += (size_t)A.cap_ff * n;
    L.fw = p;
    p += (size_t)A.cap_fw * n;
    L.wf = p;
    p += (size_t)A.cap_wf * nw;
    L.ffc = p;
    p += n;
    L.fwc = p;
    p += n;
    L.wfc = p;
    return L;
}
template <typename T>
WallSet<T> seg_walls(const AdjointState& A, long long steps, long long k) {
    const size_t nw = (size_t)std::max(A.nw, 1);
    const size_t lists = ((list_set_ints(A) * 4 + 255) / 256) * 256;
    const size_t walls = ((wall_set_elems<T>(A) * sizeof(T) + 255) / 256) * 256;
    T* p = (T*)((char*)A.seg + (size_t)steps * lists + (size_t)k * walls);
    WallSet<T> W;
    W.pf = p;
    p += A.nf;
    W.wp = p;
    p += nw;
    W.wr = p;
    p += nw;
    W.wnum = p;
    p += nw;
    W.wvol = p;
    return W;
}

template <typename T>
AdjLam<T> lam_of(const AdjointState& A) {
    const size_t n = (size_t)A.nf, nd = (size_t)A.nd, nw = (size_t)std::max(A.nw, 1);
    T* p = (T*)A.lam;
    AdjLam<T> L;
    L.x = p;
    p += n * nd;
    L.v = p;
    p += n * nd;
    L.r = p;
    p += n;
    L.p = p;
    p += n;
    L.dx = p;
    p += n * nd;
    L.dv = p;
    p += n * nd;
    L.dr = p;
    p += n;
    L.fv = p;
    p += n * nd;
    L.fr = p;
    p += n;
    L.wp = p;
    p += nw;
    L.wr = p;
    return L;
}

template <typename T>
size_t lam_elems(const AdjointState& A) {
    const size_t n = (size_t)A.nf, nd = (size_t)A.nd, nw = (size_t)std::max(A.nw, 1);
    return n * (5 * nd + 5) + 2 * nw;
}

void free_all(AdjointState* A) {
    void* ptrs[] = {A->ff, A->fw, A->wf, A->ffc, A->fwc, A->wfc, A->xb, A->mf, A->pf, A->wp,
                    A->wr, A->wnum, A->wvol, A->tx, A->tv, A->tr, A->pingpong, A->ckpt, A->tape,
                    A->lam, A->theta, A->seg};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (A->h_theta) cudaFreeHost(A->h_theta);
}

template <class P>
cudaError_t dmalloc(P** p, size_t bytes) {
    *p = nullptr;
    return cudaMalloc((void**)p, std::max<size_t>(bytes, 16));
}

int list_capacity(int nd, double skin, int maxcell) {
    const double q = 1.0 + skin;
    const double ball = (nd == 3) ? (4.0 / 3.0) * 3.141592653589793 * q * q * q
                                  : 3.141592653589793 * q * q;
    // room for twice the densest cell seen at the start (the lists are not re-sized later)
    const double c = std::ceil(1.3 * ball * 2.0 * (double)std::max(maxcell, 1)) + 32.0;
    return ((int)c + 31) / 32 * 32;
}

// Allocation of everything but checkpoints and tape (sized per forward call).
template <typename T>
tp_status ensure_adjoint(tp_handle* h, const double* u) {
    AdjointState*& A = h->adj;
    if (A && A->f32 != (sizeof(T) == 4)) {
        free_all(A);
        delete A;
        A = nullptr;
    }
    if (!A) {
        A = new AdjointState();
        A->f32 = sizeof(T) == 4;
        A->nd = h->cfg.ndims;
        A->nf = (int)h->cfg.n_fluid;
        A->nw = (int)h->cfg.n_wall;
        const size_t n = (size_t)A->nf, nd = (size_t)A->nd, nw = (size_t)std::max(A->nw, 1);
        ADJ_CUDA(h, dmalloc(&A->ffc, n * 4));
        ADJ_CUDA(h, dmalloc(&A->fwc, n * 4));
        ADJ_CUDA(h, dmalloc(&A->wfc, nw * 4));
        ADJ_CUDA(h, dmalloc(&A->xb, n * nd * 8));
        ADJ_CUDA(h, dmalloc(&A->mf, n * sizeof(T)));
        ADJ_CUDA(h, dmalloc(&A->pf, n * sizeof(T)));
        ADJ_CUDA(h, dmalloc(&A->wp, nw * sizeof(T)));
        ADJ_CUDA(h, dmalloc(&A->wr, nw * sizeof(T)));
        ADJ_CUDA(h, dmalloc(&A->wnum, nw * sizeof(T)));
        ADJ_CUDA(h, dmalloc(&A->wvol, nw * sizeof(T)));
        ADJ_CUDA(h, dmalloc(&A->tx, n * nd * 8));
        ADJ_CUDA(h, dmalloc(&A->tv, n * nd * sizeof(T)));
        ADJ_CUDA(h, dmalloc(&A->tr, n * sizeof(T)));
        ADJ_CUDA(h, dmalloc(&A->pingpong, 2 * state_bytes<T>(*A)));
        ADJ_CUDA(h, dmalloc(&A->lam, lam_elems<T>(*A) * sizeof(T)));
        ADJ_CUDA(h, dmalloc(&A->theta, 3 * sizeof(double)));
        ADJ_CUDA(h, cudaMallocHost((void**)&A->h_theta, 3 * sizeof(double)));
    }
    // list capacities from the densest fluid cell of the initial coordinates (one sync)
    ADJ_CUDA(h, cudaMemsetAsync(h->d_max, 0, sizeof(int), h->stream));
    tp_status st = sort_fluid_cells(h, u, h->d_max);
    if (st != TP_OK) return st;
    int maxcell = 0;
    ADJ_CUDA(h, cudaMemcpyAsync(&maxcell, h->d_max, sizeof(int), cudaMemcpyDeviceToHost,
                                h->stream));
    ADJ_CUDA(h, cudaStreamSynchronize(h->stream));
    const int cff = list_capacity(A->nd, A->skin, maxcell);
    const int cfw = list_capacity(A->nd, A->skin, h->maxcell_w);
    auto grow = [&](int** buf, int* cap, int want, int rows) -> cudaError_t {
        if (*cap >= want && *buf) return cudaSuccess;
        if (*buf) cudaFree(*buf);
        *buf = nullptr;
        *cap = 0;
        cudaError_t e = dmalloc(buf, (size_t)want * (size_t)std::max(rows, 1) * 4);
        if (e == cudaSuccess) *cap = want;
        return e;
    };
    ADJ_CUDA(h, grow(&A->ff, &A->cap_ff, cff, A->nf));
    ADJ_CUDA(h, grow(&A->fw, &A->cap_fw, cfw, A->nf));
    ADJ_CUDA(h, grow(&A->wf, &A->cap_wf, cff, A->nw));
    return TP_OK;
}

template <int ND>
tp_status build_lists_at(tp_handle* h, const double* x, const ListSet& L) {
    AdjointState& A = *h->adj;
    tp_status st = sort_fluid_cells(h, x, nullptr);
    if (st != TP_OK) return st;
    const double r = 2.0 * h->cfg.smoothing_length * (1.0 + A.skin);
    const double rl2 = r * r;
    const double m = r - h->grid.cs;
    if (A.nf > 0)
        k_adj_fluid_lists<ND><<<nb(A.nf, 128), 128, 0, h->stream>>>(
            h->grid, rl2, m, A.nf, x, h->f_key, h->f_start, h->f_perm,
            (const double4_32a*)h->w_pos, h->w_start, L.ff, L.ffc, A.cap_ff, L.fw, L.fwc, A.cap_fw,
            A.xb, h->d_err);
    if (A.nw > 0)
        k_adj_wall_lists<ND><<<nb(A.nw, 128), 128, 0, h->stream>>>(
            h->grid, rl2, m, A.nw, (const double4_32a*)h->w_pos, h->w_skey, x, h->f_start,
            h->f_perm, L.wf, L.wfc, A.cap_wf, h->d_err);
    ADJ_LAUNCHED(h, "adjoint lists");
    A.kernels += 2;
    return TP_OK;
}

// Pressure + Adami of state s over the wall lists of L, into W.
template <typename T, int ND>
tp_status wall_state(tp_handle* h, const AdjPhys<T>& P, AState<T> s, const ListSet& L,
                     const WallSet<T>& W) {
    AdjointState& A = *h->adj;
    k_adj_pressure<T><<<nb(A.nf, 256), 256, 0, h->stream>>>(P, s.r, W.pf, A.nf);
    if (A.nw > 0)
        k_adj_adami<T, ND><<<nb((long)A.nw * kAdjLanes, 128), 128, 0, h->stream>>>(
            P, A.nw, (const double4_32a*)h->w_pos, L.wf, L.wfc, s, (const T*)W.pf, W.wp, W.wr,
            W.wnum, W.wvol);
    ADJ_LAUNCHED(h, "adjoint wall state");
    A.kernels += 1 + (A.nw > 0);
    return TP_OK;
}

// One CK2N54 step from state `from` using `scratch` as the ping-pong partner; the result lands
// in `out`.  With `tape` non-null the five stage inputs are tape[0..4] (tape[0] = from) and the
// result is tape[5].  `lists` (optional) receives the step's neighbour lists and `walls`
// (optional, five entries) the pressure / wall state of each stage; by default both go to the
// handle's working arrays.
template <typename T, int ND>
tp_status forward_step(tp_handle* h, const AdjPhys<T>& P, double dt, AState<T> from,
                       AState<T> other, AState<T>* tape, AState<T>* out,
                       const ListSet* lists = nullptr, const WallSet<T>* walls = nullptr) {
    AdjointState& A = *h->adj;
    const ListSet L = lists ? *lists : lists_of(A);
    tp_status st = build_lists_at<ND>(h, from.x, L);
    if (st != TP_OK) return st;
    AState<T> src = from;
    for (int i = 0; i < 5; ++i) {
        AState<T> dst = tape ? tape[i + 1] : ((i % 2 == 0) ? other : from);
        const WallSet<T> W = walls ? walls[i] : walls_of<T>(A);
        st = wall_state<T, ND>(h, P, src, L, W);
        if (st != TP_OK) return st;
        AdjStage<T> S;
        S.A = (T)kCK2N54_A[i];
        S.B = (T)kCK2N54_B[i];
        S.dt = (T)dt;
        S.Ad = kCK2N54_A[i];
        S.Bd = kCK2N54_B[i];
        S.dtd = dt;
        S.first = i == 0;
        k_adj_stage<T, ND><<<nb((long)A.nf * kAdjLanes, 128), 128, 0, h->stream>>>(
            P, A.nf, src, dst, (const T*)W.pf, (const T*)A.mf, L.ff, L.ffc, L.fw, L.fwc,
            (const double4_32a*)h->w_pos, (const T*)W.wp, (const T*)W.wr, A.tx, (T*)A.tv,
            (T*)A.tr, S);
        ADJ_LAUNCHED(h, "adjoint forward stage");
        A.kernels += 1;
        src = dst;
    }
    k_adj_skin_check<ND><<<nb(A.nf, 256), 256, 0, h->stream>>>(
        src.x, A.xb, A.nf, (A.skin * h->cfg.smoothing_length) * (A.skin * h->cfg.smoothing_length),
        h->d_err);
    ADJ_LAUNCHED(h, "adjoint skin check");
    A.kernels += 1;
    *out = src;
    return TP_OK;
}

tp_status read_errors(tp_handle* h) {
    ADJ_CUDA(h, cudaMemcpyAsync(h->h_err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost,
                                h->stream));
    ADJ_CUDA(h, cudaStreamSynchronize(h->stream));
    const int bits = *h->h_err;
    if (!bits) return TP_OK;
    *h->h_err = 0;
    ADJ_CUDA(h, cudaMemset(h->d_err, 0, sizeof(int)));
    if (bits & TP_ERRBIT_NONFINITE)
        return api_fail(h, TP_ERR_NONFINITE, "a particle coordinate became NaN or Inf");
    if (bits & kAdjErrSkin)
        return api_fail(h, TP_ERR_CAPACITY,
                        "a particle moved more than the list skin (0.1 h) within one step: "
                        "the time step is too large for the fixed per-step neighbour lists");
    if (bits & TP_ERRBIT_CAPACITY)
        return api_fail(h, TP_ERR_CAPACITY, "a neighbour list of the adjoint overflowed");
    return api_fail(h, TP_ERR_OUT_OF_GRID,
                    "a particle left the FullGridCellList bounding box (its cell was clamped)");
}

template <typename T, int ND>
tp_status forward_impl(tp_handle* h, double* v_ode, double* u_ode, double dt, long long n_steps,
                       long long every) {
    tp_status st = ensure_adjoint<T>(h, u_ode);
    if (st != TP_OK) return st;
    AdjointState& A = *h->adj;
    A.recorded = false;
    const size_t sb = state_bytes<T>(A);
    const size_t n_ckpt = (size_t)((n_steps + every - 1) / every);
    if (A.n_ckpt < n_ckpt) {
        if (A.ckpt) cudaFree(A.ckpt);
        A.ckpt = nullptr;
        A.n_ckpt = 0;
        ADJ_CUDA(h, dmalloc(&A.ckpt, n_ckpt * sb));
        A.n_ckpt = n_ckpt;
    }
    const size_t n_tape = (size_t)(5 * std::min(every, n_steps) + 1);
    if (A.n_tape < n_tape) {
        if (A.tape) cudaFree(A.tape);
        A.tape = nullptr;
        A.n_tape = 0;
        ADJ_CUDA(h, dmalloc(&A.tape, n_tape * sb));
        A.n_tape = n_tape;
    }
    const AdjPhys<T> P = make_phys<T>(h);
    AState<T> s0 = state_at<T>(A, A.pingpong, 0), s1 = state_at<T>(A, A.pingpong, 1);
    k_adj_load<T, ND><<<nb(A.nf, 256), 256, 0, h->stream>>>(v_ode, u_ode, h->m_f,
                                                            h->cfg.reference_density, s0,
                                                            (T*)A.mf, A.nf);
    ADJ_LAUNCHED(h, "adjoint load");
    AState<T> cur = s0, oth = s1;
    for (long long step = 0; step < n_steps; ++step) {
        if (step % every == 0) {
            k_adj_copy<T, ND><<<nb(A.nf, 256), 256, 0, h->stream>>>(
                cur, state_at<T>(A, A.ckpt, (size_t)(step / every)), A.nf);
            ADJ_LAUNCHED(h, "adjoint checkpoint");
        }
        AState<T> out;
        st = forward_step<T, ND>(h, P, dt, cur, oth, nullptr, &out);
        if (st != TP_OK) return st;
        // five stages alternate from->other->from->other->from->other: the result is in `other`
        oth = cur;
        cur = out;
    }
    k_adj_store<T, ND><<<nb(A.nf, 256), 256, 0, h->stream>>>(cur, h->cfg.reference_density,
                                                             v_ode, u_ode, A.nf);
    ADJ_LAUNCHED(h, "adjoint store");
    st = read_errors(h);
    if (st != TP_OK) return st;
    A.recorded = true;
    A.dt = dt;
    A.n_steps = n_steps;
    A.every = every;
    return TP_OK;
}

template <typename T, int ND>
tp_status backward_impl(tp_handle* h, double* v_bar, double* u_bar, double* params_bar) {
    AdjointState& A = *h->adj;
    const AdjPhys<T> P = make_phys<T>(h);
    const AdjLam<T> L = lam_of<T>(A);
    k_adj_lam_load<T, ND><<<nb(A.nf, 256), 256, 0, h->stream>>>(v_bar, u_bar, L, A.nf);
    ADJ_CUDA(h, cudaMemsetAsync(A.theta, 0, 3 * sizeof(double), h->stream));
    ADJ_LAUNCHED(h, "adjoint seed load");
    std::vector<AState<T>> tape(A.n_tape);
    for (size_t k = 0; k < A.n_tape; ++k) tape[k] = state_at<T>(A, A.tape, k);
    // segment storage for the lists and wall states of the recomputation (used when it takes at
    // most a quarter of the free device memory; otherwise the reverse sweep rebuilds them)
    const long long seg_steps = std::min(A.every, A.n_steps);
    const size_t want = seg_bytes_for<T>(A, seg_steps);
    if (A.seg_bytes < want) {
        if (A.seg) cudaFree(A.seg);
        A.seg = nullptr;
        A.seg_bytes = 0;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && want <= free_b / 4 &&
            dmalloc(&A.seg, want) == cudaSuccess)
            A.seg_bytes = want;
        else
            cudaGetLastError();  // a refused allocation only selects the rebuilding path
    }
    const bool keep = A.seg != nullptr;
    std::vector<ListSet> seg_l;
    std::vector<WallSet<T>> seg_w;
    if (keep) {
        for (long long j = 0; j < seg_steps; ++j) seg_l.push_back(seg_lists(A, j));
        for (long long k = 0; k < 5 * seg_steps; ++k) seg_w.push_back(seg_walls<T>(A, seg_steps, k));
    }
    const long long n_seg = (A.n_steps + A.every - 1) / A.every;
    for (long long seg = n_seg - 1; seg >= 0; --seg) {
        const long long s0 = seg * A.every;
        const long long ns = std::min(A.every, A.n_steps - s0);
        // recompute the segment, recording every stage input (and, with segment storage, the
        // lists of every step and the wall state of every stage)
        k_adj_copy<T, ND><<<nb(A.nf, 256), 256, 0, h->stream>>>(
            state_at<T>(A, A.ckpt, (size_t)seg), tape[0], A.nf);
        ADJ_LAUNCHED(h, "adjoint restore");
        for (long long j = 0; j < ns; ++j) {
            AState<T> out;
            tp_status st = forward_step<T, ND>(h, P, A.dt, tape[5 * j], tape[5 * j], &tape[5 * j],
                                               &out, keep ? &seg_l[j] : nullptr,
                                               keep ? &seg_w[5 * j] : nullptr);
            if (st != TP_OK) return st;
        }
        // reverse the segment's steps and stages
        for (long long j = ns - 1; j >= 0; --j) {
            const ListSet LS = keep ? seg_l[j] : lists_of(A);
            if (!keep) {
                tp_status st = build_lists_at<ND>(h, tape[5 * j].x, LS);
                if (st != TP_OK) return st;
            }
            for (int i = 4; i >= 0; --i) {
                const AState<T> U = tape[5 * j + i];
                const WallSet<T> W = keep ? seg_w[5 * j + i] : walls_of<T>(A);
                if (!keep) {
                    tp_status st = wall_state<T, ND>(h, P, U, LS, W);
                    if (st != TP_OK) return st;
                }
                k_adj_seed<T, ND><<<nb(std::max(A.nf, A.nw), 256), 256, 0, h->stream>>>(
                    L, (T)kCK2N54_A[i], (T)kCK2N54_B[i], (T)A.dt, A.nf, A.nw);
                k_adj_pair_vjp<T, ND><<<nb((long)A.nf * kAdjLanes, 128), 128, 0, h->stream>>>(
                    P, A.nf, U, (const T*)W.pf, (const T*)A.mf, LS.ff, LS.ffc, LS.fw, LS.fwc,
                    (const double4_32a*)h->w_pos, (const T*)W.wp, (const T*)W.wr, L, A.theta);
                if (A.nw > 0)
                    k_adj_adami_vjp<T, ND><<<nb((long)A.nw * kAdjLanes, 128), 128, 0,
                                             h->stream>>>(
                        P, A.nw, (const double4_32a*)h->w_pos, LS.wf, LS.wfc, U, (const T*)W.pf,
                        (const T*)W.wp, (const T*)W.wnum, (const T*)W.wvol, L, A.theta);
                k_adj_eos_vjp<T><<<nb(A.nf, 256), 256, 0, h->stream>>>(P, U.r, L, A.nf);
                ADJ_LAUNCHED(h, "adjoint stage");
                A.kernels += 3 + (A.nw > 0);
            }
        }
    }
    k_adj_lam_store<T, ND><<<nb(A.nf, 256), 256, 0, h->stream>>>(L, v_bar, u_bar, A.nf);
    ADJ_LAUNCHED(h, "adjoint store");
    ADJ_CUDA(h, cudaMemcpyAsync(A.h_theta, A.theta, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                h->stream));
    tp_status st = read_errors(h);  // synchronises
    if (st != TP_OK) return st;
    for (int k = 0; k < 3; ++k) params_bar[k] = A.h_theta[k];
    return TP_OK;
}

}  // namespace

void adjoint_release(tp_handle* h) {
    if (!h || !h->adj) return;
    free_all(h->adj);
    delete h->adj;
    h->adj = nullptr;
}

}  // namespace tp

using namespace tp;

extern "C" {

tp_status tp_adjoint_forward(tp_handle* h, double* v_ode, double* u_ode, double dt,
                             int64_t n_steps, int64_t checkpoint_every) {
    if (!h) return TP_ERR_ARGUMENT;
    if (!h->wall_set || !h->mass_set)
        return api_fail(h, TP_ERR_NOT_READY, "tp_adjoint_forward: wall or masses not set");
    if (n_steps <= 0 || checkpoint_every <= 0 || !(dt > 0.0) || !std::isfinite(dt))
        return api_fail(h, TP_ERR_ARGUMENT,
                        "tp_adjoint_forward: n_steps, checkpoint_every and dt must be positive");
    if (h->cfg.n_fluid == 0 || !v_ode || !u_ode)
        return api_fail(h, TP_ERR_ARGUMENT, "tp_adjoint_forward: empty fluid or null array");
    const bool f32 = h->cfg.precision == TP_PRECISION_FP32;
    if (h->cfg.ndims == 2)
        return f32 ? forward_impl<float, 2>(h, v_ode, u_ode, dt, n_steps, checkpoint_every)
                   : forward_impl<double, 2>(h, v_ode, u_ode, dt, n_steps, checkpoint_every);
    return f32 ? forward_impl<float, 3>(h, v_ode, u_ode, dt, n_steps, checkpoint_every)
               : forward_impl<double, 3>(h, v_ode, u_ode, dt, n_steps, checkpoint_every);
}

tp_status tp_adjoint_backward(tp_handle* h, double* v_bar, double* u_bar, double params_bar[3]) {
    if (!h) return TP_ERR_ARGUMENT;
    if (!h->adj || !h->adj->recorded)
        return api_fail(h, TP_ERR_NOT_READY, "tp_adjoint_backward: no recorded forward");
    if (!v_bar || !u_bar || !params_bar)
        return api_fail(h, TP_ERR_ARGUMENT, "tp_adjoint_backward: null array");
    const bool f32 = h->adj->f32;
    if (h->cfg.ndims == 2)
        return f32 ? backward_impl<float, 2>(h, v_bar, u_bar, params_bar)
                   : backward_impl<double, 2>(h, v_bar, u_bar, params_bar);
    return f32 ? backward_impl<float, 3>(h, v_bar, u_bar, params_bar)
               : backward_impl<double, 3>(h, v_bar, u_bar, params_bar);
}

int64_t tp_adjoint_kernel_launches(const tp_handle* h) {
    return (h && h->adj) ? (int64_t)h->adj->kernels : 0;
}

}  // extern "C"
