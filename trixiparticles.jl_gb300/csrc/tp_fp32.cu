// tp_fp32.cu — FP32 precision form of the WCSPH right-hand side (sm_103a).
//
// Same passes, lists and neighbour order as the FP64 drop-in, with these precision choices:
//   * positions enter the pair arithmetic as FP32 offsets inside a reference cell (the cell at
//     the last list rebuild), o = x - (cmin + c) * cs32 (FP64 on input, rounded once to FP32),
//     and a pair difference is (o_a - o_b) - (c_b - c_a) * cs32 with the cell offset taken from
//     the list entry, so it stays accurate to FP32 relative precision of h whatever the domain
//     size;
//   * density is stored as the deviation rho - rho0 in FP32, so differences of densities and
//     the Cole EOS, evaluated as B * expm1(gamma * log1p((rho - rho0) / rho0)), do not cancel;
//   * per-particle sums (dv, drho, Adami pressure and volume) use Kahan-compensated FP32;
//   * `div_fast` divisions use __fdividef, the CUDA Float32 fast division the reference's
//     Float32 GPU path compiles to;
//   * positions and their Runge-Kutta register stay FP64 (the drift! accumulation); velocity
//     and density registers are FP32.
// The neighbour set is the FP32 one: |o_a - o_b + shift|^2 <= (2h)^2 evaluated in FP32.
// A neighbour gather is 36 bytes from three slot-ordered arrays (test {offsets, rho - rho0},
// velocity {v, m / rho}, pressure): neighbouring lanes gather nearby slots, so small records keep
// many of them in one cache line.
#include "tp_api_internal.h"
#include "tp_lists.cuh"

namespace tp {

struct Kahan {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

__device__ __forceinline__ float eos32(float drho, const Phys32& P, int clip) {
    float p = P.B * expm1f(P.gamma * log1pf(drho / P.rho0)) + P.p_bg;
    if (clip) p = (p != p || p > 0.0f) ? p : 0.0f;
    return p;
}

__device__ __forceinline__ float eos32_inverse_dev(float p, const Phys32& P) {
    return P.rho0 * expm1f(log1pf((p - P.p_bg) / P.B) * P.inv_gamma);
}

// Source state -> fluid record slot.  SRC32: the integrator's FP32 velocity/density state
// (float4 {v, rho - rho0}) and FP32 masses; otherwise the caller's FP64 v_ode and masses.
template <int ND, bool SRC32>
struct Pack32 {
    const double* u;
    const void* v;
    const void* m;
    const double* tu;
    const float4* tv;
    const int* id_in;
    double* u_out;  // integrator: FP64 positions moved to slot order
    double* tu_out;
    float4* tv_out;
    int* id_out;
    float* m_out;
    double* xb_out;
    float4* test;  // {ox, oy, oz, rho - rho0}
    float4* vel;   // {vx, vy, vz, m / rho}
    float* pres;   // p
    const int* src_perm;  // kick! path: without a rebuild, slot s packs caller particle perm[s]
    GridDesc g;
    double cs32, rho0;
    Phys32 P;
    __device__ void operator()(int i, int s, int key, bool rebuild) const {
        if (!rebuild && src_perm) i = src_perm[s];
        double x[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < ND; ++d) x[d] = u[(size_t)i * ND + d];
        float4 w;
        float mi;
        if (SRC32) {
            w = ((const float4*)v)[i];
            mi = ((const float*)m)[i];
        } else {
            const double* vv = (const double*)v + (size_t)i * (ND + 1);
            w.x = (float)vv[0];
            w.y = (float)vv[1];
            w.z = (ND == 3) ? (float)vv[2] : 0.0f;
            w.w = (float)(vv[ND] - rho0);
            mi = (float)((const double*)m)[i];
        }
        // offsets against the reference cell `key` (the cell of the last rebuild); the records
        // hold what a neighbour gather needs and nothing else: 36 bytes per pair
        float4 t = test_record_in<ND>(x, g, cs32, key);
        t.w = w.w;
        test[s] = t;
        const float irho = __frcp_rn(P.rho0 + w.w);
        vel[s] = make_float4(w.x, w.y, w.z, mi * irho);
        pres[s] = eos32(w.w, P, P.fluid_clip);
        if (rebuild && xb_out) {
#pragma unroll
            for (int d = 0; d < ND; ++d) xb_out[(size_t)s * ND + d] = x[d];
        }
        if (u_out) {
            // the integrator state moves with a rebuild; without one the pair pass reads the
            // source state in place and writes the destination, so only ids and masses follow
            if (rebuild) {
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    u_out[(size_t)s * ND + d] = x[d];
                    tu_out[(size_t)s * ND + d] = tu[(size_t)i * ND + d];
                }
                tv_out[s] = tv[i];
            }
            id_out[s] = id_in[i];
            m_out[s] = mi;
        }
    }
};

// FP32 wall state: {p, rho - rho0, m, m / rho}; masses are set once, the rest by the Adami pass.
__global__ void k_wall_state32_init(const double4_32a* __restrict__ wpos, float4* __restrict__ st,
                                    int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) st[s] = make_float4(0.0f, 0.0f, (float)wpos[s].w, 0.0f);
}

// Per wall slot over its fluid list: the fluid neighbour's offsets and rho - rho0 come with its
// test record, its pressure from the dense pressure array (20 bytes per pair).  Besides the wall
// state, the pass leaves m / rho of the wall in the fourth slot of its test record and its
// pressure in a dense array, which is what the fluid pair pass gathers.
template <int ND>
__global__ void __launch_bounds__(256) k_adami32(Phys32 P, int nw, float4* __restrict__ wtest,
                                                 const unsigned* __restrict__ wf,
                                                 const int* __restrict__ wfc,
                                                 float4* __restrict__ wstate,
                                                 float* __restrict__ wpres,
                                                 double* __restrict__ wvol,
                                                 const float4* __restrict__ ftest,
                                                 const float* __restrict__ fpres) {
    __shared__ float4 off[kOffsetCodes];
    fill_offset_table(off, P.cs);
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    const float4 tw = wtest[w];
    Kahan Ps, V;
    const int n = wfc[w];
    uint4 lq;  // the list quad holding entry k
    for (int k = 0; k < n; ++k) {
        const unsigned e = list_next(wf, k, nw, w, lq);
        const int b = (int)(e & kSlotMask);
        const float4 cb = ftest[b];
        float pd0, pd1, pd2;
        const float d2 = pair_diff<ND>(tw, off, e, cb, pd0, pd1, pd2);
        if (d2 > P.sr2) continue;
        const float r = sqrtf(d2);
        const float rho_f = P.rho0 + cb.w;
        float hp = P.g[0] * (rho_f * pd0) + P.g[1] * (rho_f * pd1);
        if (ND == 3) hp += P.g[2] * (rho_f * pd2);
        const float sum = (P.p_off + fpres[b]) + hp;
        float W = 0.0f;
        if (r < P.two_h) {
            const float q = r * P.h_inv;
            const float t = 1.0f - 0.5f * q;
            const float t2 = t * t;
            W = (P.wc2_norm * (t2 * t2)) * (2.0f * q + 1.0f);
        }
        Ps.add(sum * W);
        V.add(W);
    }
    float pw = Ps.s - Ps.c;
    const float vw = V.s - V.c;
    if ((double)vw > 2.220446049250313e-16) pw = pw / vw;
    if (P.wall_clip) pw = (pw != pw || pw > 0.0f) ? pw : 0.0f;
    const float m = wstate[w].z;
    const float dr = eos32_inverse_dev(pw, P);
    const float vol = m * __frcp_rn(P.rho0 + dr);
    wstate[w] = make_float4(pw, dr, m, vol);  // {p, rho - rho0, m, m/rho}
    wpres[w] = pw;
    wtest[w].w = vol;
    wvol[w] = (double)vw;
}

struct Update32 {
    double* dv;       // kick: dv_ode (caller order, FP64) indexed by perm
    const int* perm;
    double g[3];
    // integrator (slot order): the destination state; the pass reads the positions and
    // registers from it when this stage's pack moved the state there (a rebuild), else from the
    // source state in place
    double* u;
    double* tu;
    float4* v_out;
    float4* tv;
    const double* u_in;
    const double* tu_in;
    const float4* tv_in;
    // displacement check of the next stage (optional): positions of the last rebuild (slot
    // order) and the gate word that collects the largest squared displacement
    const double* xb;
    unsigned* gate_next;
    double A, B, dt;
    float Af, Bf, dtf;
    int first;
};

// Pair terms with the same identities as the FP64 kernels (grad W_ab = sg x_ab: one scalar for
// pressure + viscosity, continuity through sg (v_ab . x_ab), diffusion as 2 (rho_a - rho_b) sg,
// one reciprocal for the Monaghan mu / rho_mean), in FP32 on the cell-relative differences, with
// Kahan-compensated per-particle sums.
// Five 256-thread blocks per SM cap the kernel at 48 registers: the pass is bound by the L1 data
// pipe serving its neighbour gathers and by their latency, and the extra resident warps (66 %
// occupancy instead of 53 % at 56 registers) hide more of it (8 % faster at dx = 0.0064 in 3D).
// The list is read four entries per 16-byte load (the chunked layout of tp_lists.cuh).
// STD: the configuration of the dam-break setups (Monaghan viscosity with beta = 0, Molteni-
// Colagrossi diffusion) with the model switches resolved at compile time; the pass is issue
// bound, and the per-pair tests of the runtime switches are instructions of their own.
template <int ND, bool INTEGRATE, bool STD>
__global__ void __launch_bounds__(256, 5) k_pair32(Phys32 P, int nf,
                                                const float4* __restrict__ ftest,
                                                const float4* __restrict__ fvel,
                                                const float* __restrict__ fpres,
                                                const unsigned* __restrict__ ff,
                                                const int* __restrict__ ffc,
                                                const unsigned* __restrict__ fw,
                                                const int* __restrict__ fwc,
                                                const float4* __restrict__ wtest,
                                                const float* __restrict__ wpres,
                                                unsigned* __restrict__ gate, Update32 U) {
    __shared__ float4 off[kOffsetCodes];
    fill_offset_table(off, P.cs);
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    const float4 ta = ftest[s];  // {offsets, rho - rho0}
    const float4 va = fvel[s];   // {v, m / rho}
    const float p_a = fpres[s];
    const float drho_a = ta.w;
    const float rho_a = P.rho0 + drho_a;
    const float ia = __frcp_rn(rho_a);  // the pack's 1 / rho

    Kahan a0, a1, a2, ar;
    const int nff = ffc[s];
    uint4 lq;  // the list quad holding entry k
    for (int k = 0; k < nff; ++k) {
        const unsigned e = list_next(ff, k, nf, s, lq);
        const int b = (int)(e & kSlotMask);
        const float4 cb = ftest[b];  // {offsets, rho_b - rho0}
        float pd0, pd1, pd2;
        const float d2 = pair_diff<ND>(ta, off, e, cb, pd0, pd1, pd2);
        if (d2 > P.sr2 || d2 < P.az2) continue;
        const float r = d2 * rsqrtf(d2);
        const float4 vb = fvel[b];  // {v_b, m_b / rho_b}
        const float p_b = fpres[b];
        const float vol_b = vb.w;
        const float t = fmaf(-r, P.half_hinv, 1.0f);
        const float sg = P.sg_c * ((t * t) * t);
        const float vd0 = va.x - vb.x, vd1 = va.y - vb.y;
        const float vd2 = (ND == 3) ? va.z - vb.z : 0.0f;
        float vr = vd0 * pd0 + vd1 * pd1;
        if (ND == 3) vr += vd2 * pd2;
        float c = -(vol_b * ia) * (p_a + p_b);
        if ((STD || P.visc) && vr < 0.0f) {
            const float rho_b = P.rho0 + cb.w;
            const float m_b = vol_b * rho_b;
            const float den = d2 + P.visc_eps_h2;
            const float rm = 0.5f * (rho_a + rho_b);
            const float R = __fdividef(1.0f, den * rm);
            if (STD || P.beta == 0.0f) {
                c += (m_b * P.visc_k) * vr * R;
            } else {
                const float mu = (P.visc_h * vr) * (rm * R);
                c += (m_b * mu) * (P.visc_ac + P.beta * mu) * (den * R);
            }
        }
        c *= sg;
        a0.add(c * pd0);
        a1.add(c * pd1);
        if (ND == 3) a2.add(c * pd2);
        float er = (rho_a * vol_b) * (sg * vr);
        if (STD || P.diff) er += (vol_b * (drho_a - cb.w)) * (sg * P.diff2);
        ar.add(er);
    }

    Kahan w0, w1, w2, wr;
    const int nfw = fwc[s];
    for (int k = 0; k < nfw; ++k) {
        const unsigned e = list_next(fw, k, nf, s, lq);
        const int b = (int)(e & kSlotMask);
        const float4 tb = wtest[b];  // {offsets, m_w / rho_w of the last Adami pass}
        float pd0, pd1, pd2;
        const float d2 = pair_diff<ND>(ta, off, e, tb, pd0, pd1, pd2);
        if (d2 > P.sr2 || d2 < P.az2) continue;
        const float r = d2 * rsqrtf(d2);
        const float vol_b = tb.w;
        const float t = fmaf(-r, P.half_hinv, 1.0f);
        const float sg = P.sg_c * ((t * t) * t);
        const float c = (-(vol_b * ia) * (p_a + wpres[b])) * sg;
        w0.add(c * pd0);
        w1.add(c * pd1);
        if (ND == 3) w2.add(c * pd2);
        float vx = va.x * pd0 + va.y * pd1;
        if (ND == 3) vx += va.z * pd2;
        wr.add((rho_a * vol_b) * (sg * vx));
    }

    double k[4];
    k[0] = (a0.value() + w0.value()) + U.g[0];
    k[1] = (a1.value() + w1.value()) + U.g[1];
    k[2] = (ND == 3) ? (a2.value() + w2.value()) + U.g[2] : 0.0;
    k[ND] = ar.value() + wr.value();

    if (!INTEGRATE) {
        const int i = U.perm[s];
#pragma unroll
        for (int d = 0; d <= ND; ++d) U.dv[(size_t)i * (ND + 1) + d] = k[d];
    } else {
        // float4 slots: velocity components 0..ND-1 and the density deviation in slot 3
        const float kv[4] = {(float)k[0], (float)k[1], ND == 3 ? (float)k[2] : 0.0f,
                             (float)k[ND]};
        const float vin[4] = {va.x, va.y, va.z, drho_a};
        const bool moved = gate_open(gate);  // this stage rebuilt (gate[0..2] are read-only here)
        const double* u_in = moved ? U.u : U.u_in;
        const double* tu_in = moved ? U.tu : U.tu_in;
        const float4 tv = (moved ? U.tv : U.tv_in)[s];
        const float tin[4] = {tv.x, tv.y, tv.z, tv.w};
        float tout[4], vout[4];
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            const bool used = (d < ND) || (d == 3);
            const float t = U.first ? U.dtf * kv[d] : fmaf(U.dtf, kv[d], U.Af * tin[d]);
            tout[d] = used ? t : 0.0f;
            vout[d] = used ? fmaf(U.Bf, t, vin[d]) : 0.0f;
        }
        U.tv[s] = make_float4(tout[0], tout[1], tout[2], tout[3]);
        U.v_out[s] = make_float4(vout[0], vout[1], vout[2], vout[3]);
        double un[ND];
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const double ku = (double)vin[d];
            const double t = U.first ? U.dt * ku : fma(U.dt, ku, U.A * tu_in[(size_t)s * ND + d]);
            U.tu[(size_t)s * ND + d] = t;
            un[d] = fma(U.B, t, u_in[(size_t)s * ND + d]);
            U.u[(size_t)s * ND + d] = un[d];
        }
        if (U.gate_next)
            gate_max_displacement(U.gate_next, displacement2<ND>(un, U.xb + (size_t)s * ND));
    }
}

// ------------------------------------------------------------------------------------------
// Host launchers
// ------------------------------------------------------------------------------------------
namespace {
inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }
}

void fp32_pack(tp_handle* h, const double* u, const double* v, const double* m,
               const PhysState* src, PhysState* dst, const unsigned* gate) {
    const int n = (int)h->cfg.n_fluid;
    if (n == 0) return;
    const double cs32 = (double)(float)h->grid.cs;
    auto run = [&](auto ndc, auto srcc) {
        constexpr int ND = decltype(ndc)::value;
        constexpr bool S32 = decltype(srcc)::value;
        Pack32<ND, S32> pk{};
        pk.u = S32 ? src->u : u;
        pk.v = S32 ? (const void*)src->v : (const void*)v;
        pk.m = S32 ? (const void*)src->m : (const void*)m;
        if (S32) {
            pk.tu = src->tu;
            pk.tv = (const float4*)src->tv;
            pk.id_in = src->id;
            pk.u_out = dst->u;
            pk.tu_out = dst->tu;
            pk.tv_out = (float4*)dst->tv;
            pk.id_out = dst->id;
            pk.m_out = (float*)dst->m;
        }
        pk.src_perm = (!S32 && gate) ? h->f_perm : nullptr;
        pk.xb_out = h->x_build;
        pk.test = h->f_test;
        pk.vel = (float4*)h->f_vel;
        pk.pres = (float*)h->f_aux;
        pk.g = h->grid;
        pk.cs32 = cs32;
        pk.rho0 = h->cfg.reference_density;
        pk.P = h->phys32;
        k_rank_pack<<<nblk(n, 256), 256, 0, h->stream>>>(h->f_tmp, h->f_key, h->f_start, n,
                                                          h->f_perm, h->f_skey, pk, gate);
    };
    const bool s32 = src != nullptr;
    if (h->cfg.ndims == 2) {
        if (s32) run(std::integral_constant<int, 2>{}, std::true_type{});
        else run(std::integral_constant<int, 2>{}, std::false_type{});
    } else {
        if (s32) run(std::integral_constant<int, 3>{}, std::true_type{});
        else run(std::integral_constant<int, 3>{}, std::false_type{});
    }
}

// The FP32 form shares the FP64 wall records (w_pos {x, y, z, m}, w_test); it only needs its
// own state array with the masses filled in.
void fp32_init_wall_state(tp_handle* h) {
    const int n = (int)h->cfg.n_wall;
    if (n == 0) return;
    k_wall_state32_init<<<nblk(n, 256), 256, 0, h->stream>>>((const double4_32a*)h->w_pos,
                                                             (float4*)h->w_state, n);
}

void fp32_adami(tp_handle* h) {
    const int nw = (int)h->cfg.n_wall;
    if (nw == 0) return;
    if (h->cfg.ndims == 2)
        k_adami32<2><<<nblk(nw, h->pair_block), h->pair_block, 0, h->stream>>>(
            h->phys32, nw, h->w_test, h->l_wf, h->c_wf, (float4*)h->w_state, h->w_p32, h->w_vol,
            h->f_test, (const float*)h->f_aux);
    else
        k_adami32<3><<<nblk(nw, h->pair_block), h->pair_block, 0, h->stream>>>(
            h->phys32, nw, h->w_test, h->l_wf, h->c_wf, (float4*)h->w_state, h->w_p32, h->w_vol,
            h->f_test, (const float*)h->f_aux);
}

template <int ND, bool INTEG>
static void launch_pair32(tp_handle* h, unsigned* gate, const Update32& U) {
    const int nf = (int)h->cfg.n_fluid;
    const Phys32& P = h->phys32;
    const bool std_cfg = P.visc && P.beta == 0.0f && P.diff;
    auto run = [&](auto stdc) {
        k_pair32<ND, INTEG, decltype(stdc)::value><<<nblk(nf, h->pair_block), h->pair_block, 0,
                                                     h->stream>>>(
            P, nf, h->f_test, (const float4*)h->f_vel, (const float*)h->f_aux, h->l_ff, h->c_ff,
            h->l_fw, h->c_fw, h->w_test, h->w_p32, gate, U);
    };
    if (std_cfg)
        run(std::true_type{});
    else
        run(std::false_type{});
}

void fp32_pair_kick(tp_handle* h, double* dv) {
    if (h->cfg.n_fluid == 0) return;
    Update32 U{};
    U.dv = dv;
    U.perm = h->f_perm;
    for (int d = 0; d < 3; ++d) U.g[d] = h->cfg.acceleration[d];
    if (h->cfg.ndims == 2)
        launch_pair32<2, false>(h, nullptr, U);
    else
        launch_pair32<3, false>(h, nullptr, U);
}

void fp32_pair_stage(tp_handle* h, const PhysState& src, PhysState& st, double A, double B,
                     double dt, int first) {
    if (h->cfg.n_fluid == 0) return;
    Update32 U{};
    U.perm = h->f_perm;
    for (int d = 0; d < 3; ++d) U.g[d] = h->cfg.acceleration[d];
    U.u = st.u;
    U.tu = st.tu;
    U.v_out = (float4*)st.v;
    U.tv = (float4*)st.tv;
    U.u_in = src.u;
    U.tu_in = src.tu;
    U.tv_in = (const float4*)src.tv;
    U.xb = h->x_build;
    U.gate_next = h->gate + 3;
    U.A = A;
    U.B = B;
    U.dt = dt;
    U.Af = (float)A;
    U.Bf = (float)B;
    U.dtf = (float)dt;
    U.first = first;
    if (h->cfg.ndims == 2)
        launch_pair32<2, true>(h, h->gate, U);
    else
        launch_pair32<3, true>(h, h->gate, U);
}

}  // namespace tp
