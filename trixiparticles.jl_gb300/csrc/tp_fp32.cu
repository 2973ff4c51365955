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
// The list pair pass gathers one 32-byte record per candidate ({offsets, rho - rho0} and
// {v, m / rho}, one sector) and recomputes the candidate's pressure from rho - rho0; it takes the
// fluid candidates two at a time through the packed FP32 instructions of sm_100+.
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

// Cole EOS on the density deviation.  With the exponent 7 (the dam-break setups) it is the
// binomial expansion (1 + d)^7 - 1 = d (7 + d (21 + d (35 + d (35 + d (21 + d (7 + d)))))) of
// d = (rho - rho0) / rho0, six FMAs without cancellation (a few ulp of the exact power); the
// pair pass evaluates it for every accepted neighbour instead of gathering the pressure, and the
// pack writes the same value for the particle itself.
__device__ __forceinline__ float eos32(float drho, const Phys32& P, int clip) {
    float p;
    if (P.gamma7) {
        const float d = drho * P.inv_rho0;
        float q = 7.0f + d;
        q = fmaf(q, d, 21.0f);
        q = fmaf(q, d, 35.0f);
        q = fmaf(q, d, 35.0f);
        q = fmaf(q, d, 21.0f);
        q = fmaf(q, d, 7.0f);
        p = fmaf(P.B * d, q, P.p_bg);
    } else {
        p = P.B * expm1f(P.gamma * log1pf(drho / P.rho0)) + P.p_bg;
    }
    if (clip) p = (p != p || p > 0.0f) ? p : 0.0f;
    return p;
}

// One 32-byte pair record {test, velocity} with a single 256-bit load (the record is 32-byte
// aligned: one sector), through the read-only path.
__device__ __forceinline__ void load_rec32(const float4* __restrict__ rec, int s, float4& t,
                                           float4& v) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(t.x), "=f"(t.y), "=f"(t.z), "=f"(t.w), "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(rec + 2 * (size_t)s));
}

// ---- two list candidates per instruction (the packed FP32 helpers of tp_lists.cuh) ----

// Pair differences o_a - o_b + (c_a - c_b) cs of two list entries (pair_diff_decoded for both
// halves: the cell offsets decoded from the entry codes as the small integers 2 - f, so that
// (o_a - d cs) is fmaf(2 - f, cs, o_a)); returns |x_ab|^2.
template <int ND>
__device__ __forceinline__ float2 pair_diff2(float4 ta, float cs, unsigned e0, unsigned e1,
                                             float4 c0, float4 c1, float2& pdx, float2& pdy,
                                             float2& pdz) {
    const float2 code = make_float2((float)(e0 >> kSlotBits), (float)(e1 >> kSlotBits));
    float2 fz = fma2(code, f2(0.04f), f2(0.02f));
    fz = make_float2(floorf(fz.x), floorf(fz.y));
    const float2 rem = fma2(f2(-25.0f), fz, code);
    float2 fy = fma2(rem, f2(0.2f), f2(0.1f));
    fy = make_float2(floorf(fy.x), floorf(fy.y));
    const float2 nfx = sub2(f2(2.0f), fma2(f2(-5.0f), fy, rem));
    const float2 nfy = sub2(f2(2.0f), fy);
    const float2 c = f2(cs);
    pdx = sub2(fma2(nfx, c, f2(ta.x)), make_float2(c0.x, c1.x));
    pdy = sub2(fma2(nfy, c, f2(ta.y)), make_float2(c0.y, c1.y));
    float2 d2 = fma2(pdy, pdy, mul2(pdx, pdx));
    pdz = f2(0.0f);
    if (ND == 3) {
        pdz = sub2(fma2(sub2(f2(2.0f), fz), c, f2(ta.z)), make_float2(c0.z, c1.z));
        d2 = fma2(pdz, pdz, d2);
    }
    return d2;
}

// eos32 of two density deviations (the same operations, so the same values).
__device__ __forceinline__ float2 eos32x2(float2 drho, const Phys32& P, int clip) {
    float2 p;
    if (P.gamma7) {
        const float2 d = mul2(drho, f2(P.inv_rho0));
        float2 q = add2(f2(7.0f), d);
        q = fma2(q, d, f2(21.0f));
        q = fma2(q, d, f2(35.0f));
        q = fma2(q, d, f2(35.0f));
        q = fma2(q, d, f2(21.0f));
        q = fma2(q, d, f2(7.0f));
        p = fma2(mul2(f2(P.B), d), q, f2(P.p_bg));
        if (clip)
            p = make_float2((p.x != p.x || p.x > 0.0f) ? p.x : 0.0f,
                            (p.y != p.y || p.y > 0.0f) ? p.y : 0.0f);
    } else {
        p = make_float2(eos32(drho.x, P, clip), eos32(drho.y, P, clip));
    }
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
    float4* rec;   // {test, vel} in one 32-byte record (the list pair pass)
    const int* src_perm;  // kick! path: without a rebuild, slot s packs caller particle perm[s]
    // integrator stages after the first: without a rebuild the previous pair stage has written
    // the records already (Update32::rec_next), so the pass packs nothing
    bool skip_in_place;
    GridDesc g;
    double cs32, rho0;
    Phys32 P;
    __device__ void operator()(int i, int s, int key, bool rebuild) const {
        if (!rebuild && skip_in_place) return;
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
        if (test) test[s] = t;  // the tiled pass's dense array (the list pass reads the records)
        const float irho = __frcp_rn(P.rho0 + w.w);
        const float4 vr = make_float4(w.x, w.y, w.z, mi * irho);
        if (vel) {  // the tiled pass's dense arrays (the list pass reads the records)
            vel[s] = vr;
            pres[s] = eos32(w.w, P, P.fluid_clip);
        }
        rec[2 * (size_t)s] = t;
        rec[2 * (size_t)s + 1] = vr;
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

// Adami terms of the fluid candidates e0 and e1 of a wall (packed FP32; `use1` false leaves the
// second half out -- its entry is then a copy of the first): with the support test d2 <= (2h)^2
// and r < 2h, ps += (p_off + p_f + g . (rho_f x_wf)) W(r) and vs += W(r), the fluid pressure from
// its rho - rho0 by the EOS the pack applies (the same value it writes).
template <int ND>
__device__ __forceinline__ void adami_pair2(const Phys32& P, float4 tw, unsigned e0, unsigned e1,
                                            bool use1, const float4* __restrict__ frec,
                                            float2& ps, float2& vs) {
    const float4 c0 = frec[2 * (size_t)(e0 & kSlotMask)];  // {offsets, rho - rho0}
    const float4 c1 = frec[2 * (size_t)(e1 & kSlotMask)];
    float2 pdx, pdy, pdz;
    const float2 d2 = pair_diff2<ND>(tw, P.cs, e0, e1, c0, c1, pdx, pdy, pdz);
    const float2 r = make_float2(sqrtf(d2.x), sqrtf(d2.y));
    const bool in0 = !(d2.x > P.sr2) && r.x < P.two_h;
    const bool in1 = use1 && !(d2.y > P.sr2) && r.y < P.two_h;
    const float2 drho = make_float2(c0.w, c1.w);
    const float2 rho_f = add2(f2(P.rho0), drho);
    float2 hp = fma2(f2(P.g[1]), mul2(rho_f, pdy), mul2(f2(P.g[0]), mul2(rho_f, pdx)));
    if (ND == 3) hp = fma2(f2(P.g[2]), mul2(rho_f, pdz), hp);
    const float2 sum = add2(add2(f2(P.p_off), eos32x2(drho, P, P.fluid_clip)), hp);
    const float2 q = mul2(r, f2(P.h_inv));
    const float2 t = fma2(f2(-0.5f), q, f2(1.0f));
    const float2 t2 = mul2(t, t);
    float2 W = mul2(mul2(f2(P.wc2_norm), mul2(t2, t2)), fma2(f2(2.0f), q, f2(1.0f)));
    W = make_float2(in0 ? W.x : 0.0f, in1 ? W.y : 0.0f);
    ps = fma2(sum, W, ps);
    vs = add2(vs, W);
}

// Per wall slot over its fluid list (the Adami gather): the list walked a quad at a time, the
// candidates two per packed instruction, each quad's partials added into Kahan-compensated sums;
// a neighbour gather is the first half of its 32-byte record: {offsets, rho - rho0}.  Besides the wall state,
// the pass leaves m / rho of the wall in the fourth slot of its test record and its pressure in
// a dense array, which is what the fluid pair pass gathers.
template <int ND>
__global__ void __launch_bounds__(256) k_adami32(Phys32 P, int nw, float4* __restrict__ wtest,
                                                 const unsigned* __restrict__ wf,
                                                 const int* __restrict__ wfc,
                                                 float4* __restrict__ wstate,
                                                 float* __restrict__ wpres,
                                                 double* __restrict__ wvol,
                                                 const float4* __restrict__ frec) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    const float4 tw = wtest[w];
    Kahan Ps, V;
    const int n = wfc[w];
    for (int k = 0; k < n; k += 4) {
        const uint4 l = list_quad_stream(wf, k, nw, w);
        const int m = n - k;  // entries of this quad that belong to the list (>= 1)
        float2 ps = f2(0.0f), vs = f2(0.0f);
        adami_pair2<ND>(P, tw, l.x, m > 1 ? l.y : l.x, m > 1, frec, ps, vs);
        if (m > 2) adami_pair2<ND>(P, tw, l.z, m > 3 ? l.w : l.z, m > 3, frec, ps, vs);
        Ps.add(ps.x + ps.y);
        V.add(vs.x + vs.y);
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


// Stage update of one fluid slot from its compensated sums: the kick! path writes dv (gravity
// added) in caller order; the integrator applies the fused CK2N54 register update (FP32
// velocity/density, FP64 positions) and takes the next stage's displacement into the gate.
template <int ND, bool INTEGRATE>
__device__ __forceinline__ void pair32_finish(const Update32& U, int s, float4 va, float drho_a,
                                              const Kahan& a0, const Kahan& a1, const Kahan& a2,
                                              const Kahan& ar, const unsigned* gate) {
    double k[4];
    k[0] = a0.value() + U.g[0];
    k[1] = a1.value() + U.g[1];
    k[2] = (ND == 3) ? a2.value() + U.g[2] : 0.0;
    k[ND] = ar.value();

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
        if (U.rec_next) {
            // the next stage's records of the new state (what its pack would write without a
            // rebuild: offsets in the slot's reference cell, rho - rho0, v, m / rho), and the id /
            // mass copy that pack would make
            const float mi = U.m_in[s];
            float4 t = test_record_in<ND>(un, U.grid, U.cs32, U.skey[s]);
            t.w = vout[3];
            U.rec_next[2 * (size_t)s] = t;
            U.rec_next[2 * (size_t)s + 1] =
                make_float4(vout[0], vout[1], vout[2], mi * __frcp_rn(U.rho0 + vout[3]));
            U.id_out[s] = U.id_in[s];
            U.m_out[s] = mi;
        }
    }
}

// Pair terms with the same identities as the FP64 kernels (grad W_ab = sg x_ab: one scalar for
// pressure + viscosity, continuity through sg (v_ab . x_ab), diffusion as 2 (rho_a - rho_b) sg,
// one reciprocal for the Monaghan mu / rho_mean), in FP32 on the cell-relative differences.
// The list is walked one quad (four entries, one 16-byte load) at a time: the four candidates'
// test records are requested together, the accepted pairs add into plain FP32 partial sums, and
// each quad's partials enter the per-particle Kahan-compensated sums (blocked compensation: a
// partial holds at most four terms, so its rounding is that of a four-term sum, and the running
// sum over the ~50 quads of a 3D particle stays compensated).
// The pass is bound by the L1 data pipe serving its neighbour gathers.  The packed form needs 64
// registers (four 256-thread blocks per SM); capped at 48 it spills and loses to the scalar form,
// which runs five blocks at 48.
// STD: the configuration of the dam-break setups (Monaghan viscosity with beta = 0, Molteni-
// Colagrossi diffusion) with the model switches resolved at compile time, and the viscosity
// switch v_ab . x_ab < 0 taken as min(v_ab . x_ab, 0) instead of a branch.
struct FluidSums {
    float x = 0.0f, y = 0.0f, z = 0.0f, r = 0.0f;
};

// The terms of one accepted fluid-fluid pair (pd = x_a - x_b, d2 = |pd|^2) into the partials.
template <int ND, bool STD>
__device__ __forceinline__ void ff_terms32(const Phys32& P, float4 va, float p_a, float rho_a,
                                           float ia, float drho_a, float pd0, float pd1,
                                           float pd2, float d2, float4 cb, float4 vb, float p_b,
                                           FluidSums& q) {
    const float r = d2 * rsqrtf(d2);
    const float vol_b = vb.w;  // m_b / rho_b
    const float t = fmaf(-r, P.half_hinv, 1.0f);
    const float sg = P.sg_c * ((t * t) * t);
    const float vd0 = va.x - vb.x, vd1 = va.y - vb.y;
    const float vd2 = (ND == 3) ? va.z - vb.z : 0.0f;
    float vr = vd0 * pd0 + vd1 * pd1;
    if (ND == 3) vr += vd2 * pd2;
    const float rho_b = P.rho0 + cb.w;
    float c = -(vol_b * ia) * (p_a + p_b);
    if (STD) {
        const float m_b = vol_b * rho_b;
        const float R = __fdividef(1.0f, (d2 + P.visc_eps_h2) * (0.5f * (rho_a + rho_b)));
        c = fmaf((m_b * P.visc_k) * fminf(vr, 0.0f), R, c);
    } else if (P.visc && vr < 0.0f) {
        const float m_b = vol_b * rho_b;
        const float den = d2 + P.visc_eps_h2;
        const float rm = 0.5f * (rho_a + rho_b);
        const float R = __fdividef(1.0f, den * rm);
        if (P.beta == 0.0f) {
            c += (m_b * P.visc_k) * vr * R;
        } else {
            const float mu = (P.visc_h * vr) * (rm * R);
            c += (m_b * mu) * (P.visc_ac + P.beta * mu) * (den * R);
        }
    }
    c *= sg;
    q.x = fmaf(c, pd0, q.x);
    q.y = fmaf(c, pd1, q.y);
    if (ND == 3) q.z = fmaf(c, pd2, q.z);
    // continuity rho_a m_b / rho_b v_ab . grad W plus the diffusion term, one factor sg m_b/rho_b
    const float dterm = (STD || P.diff) ? P.diff2 * (drho_a - cb.w) : 0.0f;
    q.r = fmaf((sg * vol_b), fmaf(rho_a, vr, dterm), q.r);
}

// The terms of one accepted fluid-wall pair (vol_b = m_w / rho_w of the last Adami pass).
template <int ND>
__device__ __forceinline__ void fw_terms32(const Phys32& P, float4 va, float p_a, float rho_a,
                                           float ia, float pd0, float pd1, float pd2, float d2,
                                           float vol_b, float p_w, FluidSums& q) {
    const float r = d2 * rsqrtf(d2);
    const float t = fmaf(-r, P.half_hinv, 1.0f);
    const float sg = P.sg_c * ((t * t) * t);
    const float c = (-(vol_b * ia) * (p_a + p_w)) * sg;
    q.x = fmaf(c, pd0, q.x);
    q.y = fmaf(c, pd1, q.y);
    if (ND == 3) q.z = fmaf(c, pd2, q.z);
    float vx = va.x * pd0 + va.y * pd1;
    if (ND == 3) vx += va.z * pd2;
    q.r = fmaf((rho_a * vol_b) * sg, vx, q.r);
}

// List entry e: the candidate's 32-byte record (test and velocity, one 256-bit load), the
// exact test on the cell-relative difference (cell offset decoded from the entry), then the
// pair terms with the candidate's pressure from its density deviation (the value the pack wrote
// for it, recomputed instead of gathered).
template <int ND, bool STD>
__device__ __forceinline__ void ff_pair32(const Phys32& P, float4 ta, float4 va, float p_a,
                                          float rho_a, float ia, float drho_a, unsigned e,
                                          const float4* __restrict__ frec, FluidSums& q) {
    float4 cb, vb;
    load_rec32(frec, (int)(e & kSlotMask), cb, vb);
    float pd0, pd1, pd2;
    const float d2 = pair_diff_decoded<ND>(ta, P.cs, e, cb, pd0, pd1, pd2);
    if (d2 > P.sr2 || d2 < P.az2) return;
    ff_terms32<ND, STD>(P, va, p_a, rho_a, ia, drho_a, pd0, pd1, pd2, d2, cb, vb,
                        eos32(cb.w, P, P.fluid_clip), q);
}

// The slot's own values, each in both halves of a pair.
struct Own2 {
    float4 t;                                       // the slot's test record
    float2 vx, vy, vz, pa, rhoa, nia, drhoa;        // nia = -1 / rho_a
};

// Partial sums of a quad: the .x halves collect the first, third candidate, the .y halves the
// second, fourth.
struct FluidSums2 {
    float2 x = {0.0f, 0.0f}, y = {0.0f, 0.0f}, z = {0.0f, 0.0f}, r = {0.0f, 0.0f};
};

// The entry that stands for "no candidate" in a packed pair: the slot itself at cell offset
// (0, 0, 0) (code 2 + 5 * 2 + 25 * 2), whose zero distance the exact test rejects.
__device__ __forceinline__ unsigned self_entry(int s) {
    return (unsigned)s | (62u << kSlotBits);
}

// ff_pair32 for the candidates e0 and e1 at once: the same terms, each half rounded as the
// scalar code rounds it; a candidate that fails the exact test contributes exact zeros (its
// kernel factor is replaced by 0 after the terms, which stay finite for any two particles).
template <int ND, bool STD>
__device__ __forceinline__ void ff_pair32x2(const Phys32& P, const Own2& A, unsigned e0,
                                            unsigned e1, const float4* __restrict__ frec,
                                            FluidSums2& q) {
    float4 c0, v0, c1, v1;
    load_rec32(frec, (int)(e0 & kSlotMask), c0, v0);
    load_rec32(frec, (int)(e1 & kSlotMask), c1, v1);
    float2 pdx, pdy, pdz;
    const float2 d2 = pair_diff2<ND>(A.t, P.cs, e0, e1, c0, c1, pdx, pdy, pdz);
    const bool ok0 = !(d2.x > P.sr2 || d2.x < P.az2);
    const bool ok1 = !(d2.y > P.sr2 || d2.y < P.az2);
    if (!(ok0 || ok1)) return;

    const float2 r = mul2(d2, make_float2(rsqrtf(d2.x), rsqrtf(d2.y)));
    const float2 t = fma2(r, f2(-P.half_hinv), f2(1.0f));
    float2 sg = mul2(f2(P.sg_c), mul2(mul2(t, t), t));
    sg = make_float2(ok0 ? sg.x : 0.0f, ok1 ? sg.y : 0.0f);
    const float2 volb = make_float2(v0.w, v1.w);  // m_b / rho_b
    const float2 drhob = make_float2(c0.w, c1.w);
    const float2 vd0 = sub2(A.vx, make_float2(v0.x, v1.x));
    const float2 vd1 = sub2(A.vy, make_float2(v0.y, v1.y));
    float2 vr = fma2(vd1, pdy, mul2(vd0, pdx));
    if (ND == 3) vr = fma2(sub2(A.vz, make_float2(v0.z, v1.z)), pdz, vr);
    const float2 rhob = add2(f2(P.rho0), drhob);
    const float2 pb = eos32x2(drhob, P, P.fluid_clip);  // the candidates' pressures
    float2 c = mul2(mul2(volb, A.nia), add2(A.pa, pb));
    if (STD) {
        const float2 mb = mul2(volb, rhob);
        const float2 x = mul2(add2(d2, f2(P.visc_eps_h2)), mul2(f2(0.5f), add2(A.rhoa, rhob)));
        const float2 R = make_float2(__fdividef(1.0f, x.x), __fdividef(1.0f, x.y));
        const float2 vneg = make_float2(fminf(vr.x, 0.0f), fminf(vr.y, 0.0f));
        c = fma2(mul2(mul2(mb, f2(P.visc_k)), vneg), R, c);
    } else if (P.visc) {
        auto visc = [&](float vr_, float d2_, float rho_b, float vol_b, float c_) {
            if (!(vr_ < 0.0f)) return c_;
            const float m_b = vol_b * rho_b;
            const float den = d2_ + P.visc_eps_h2;
            const float rm = 0.5f * (A.rhoa.x + rho_b);
            const float R = __fdividef(1.0f, den * rm);
            if (P.beta == 0.0f) return c_ + (m_b * P.visc_k) * vr_ * R;
            const float mu = (P.visc_h * vr_) * (rm * R);
            return c_ + (m_b * mu) * (P.visc_ac + P.beta * mu) * (den * R);
        };
        c = make_float2(visc(vr.x, d2.x, rhob.x, volb.x, c.x), visc(vr.y, d2.y, rhob.y, volb.y, c.y));
    }
    c = mul2(c, sg);
    q.x = fma2(c, pdx, q.x);
    q.y = fma2(c, pdy, q.y);
    if (ND == 3) q.z = fma2(c, pdz, q.z);
    const float2 dterm =
        (STD || P.diff) ? mul2(f2(P.diff2), sub2(A.drhoa, drhob)) : f2(0.0f);
    q.r = fma2(mul2(sg, volb), fma2(A.rhoa, vr, dterm), q.r);
}

template <int ND>
__device__ __forceinline__ void fw_pair32(const Phys32& P, float4 ta, float4 va, float p_a,
                                          float rho_a, float ia, unsigned e, float4 tb,
                                          const float* __restrict__ wpres, FluidSums& q) {
    float pd0, pd1, pd2;
    const float d2 = pair_diff_decoded<ND>(ta, P.cs, e, tb, pd0, pd1, pd2);
    if (d2 > P.sr2 || d2 < P.az2) return;
    fw_terms32<ND>(P, va, p_a, rho_a, ia, pd0, pd1, pd2, d2, tb.w, wpres[e & kSlotMask], q);
}

// Fluid-fluid candidates two at a time with packed FP32 instructions (ff_pair32x2) instead of one
// at a time (ff_pair32): in 3D (the 512-instance 2D ensemble measured 0.7 % faster with the scalar
// form, whose 48 registers keep five blocks per SM).
template <int ND>
constexpr bool kPackedPairs = ND == 3;

// One fluid slot s of the list pass (a thread's whole work; shared by the per-handle kernel and
// the batched persistent pass).
template <int ND, bool INTEGRATE, bool STD>
__device__ __forceinline__ void pair32_slot(const Phys32& P, int s, int nf,
                                            const float4* __restrict__ frec,
                                            const unsigned* __restrict__ ff,
                                            const int* __restrict__ ffc,
                                            const unsigned* __restrict__ fw,
                                            const int* __restrict__ fwc,
                                            const float4* __restrict__ wtest,
                                            const float* __restrict__ wpres,
                                            unsigned* __restrict__ gate, const Update32& U) {
    if (s >= nf) return;
    const float4 ta = frec[2 * (size_t)s];      // {offsets, rho - rho0}
    const float4 va = frec[2 * (size_t)s + 1];  // {v, m / rho}
    const float p_a = eos32(ta.w, P, P.fluid_clip);  // the pack's value
    const float drho_a = ta.w;
    const float rho_a = P.rho0 + drho_a;
    const float ia = __frcp_rn(rho_a);  // the pack's 1 / rho

    Kahan a0, a1, a2, ar;
    auto settle = [&](const FluidSums& q) {
        a0.add(q.x);
        a1.add(q.y);
        if (ND == 3) a2.add(q.z);
        ar.add(q.r);
    };
    const int nff = ffc[s];
    if (kPackedPairs<ND>) {
        // two candidates per packed instruction; the halves of a quad's partials are added
        // before they enter the compensated sums
        const Own2 A = {ta, f2(va.x), f2(va.y), f2(va.z), f2(p_a), f2(rho_a), f2(-ia),
                        f2(drho_a)};
        auto settle2 = [&](const FluidSums2& q2) {
            FluidSums q;
            q.x = q2.x.x + q2.x.y;
            q.y = q2.y.x + q2.y.y;
            q.z = q2.z.x + q2.z.y;
            q.r = q2.r.x + q2.r.y;
            settle(q);
        };
        for (int k = 0; k < (nff & ~3); k += 4) {
            const uint4 l = list_quad_stream(ff, k, nf, s);
            FluidSums2 q;
            ff_pair32x2<ND, STD>(P, A, l.x, l.y, frec, q);
            ff_pair32x2<ND, STD>(P, A, l.z, l.w, frec, q);
            settle2(q);
        }
        if (nff & 3) {  // the open quad: entries beyond the count are not part of the list
            const int k = nff & ~3, m = nff & 3;
            const uint4 l = list_quad_stream(ff, k, nf, s);
            const unsigned none = self_entry(s);
            FluidSums2 q;
            ff_pair32x2<ND, STD>(P, A, l.x, m > 1 ? l.y : none, frec, q);
            if (m > 2) ff_pair32x2<ND, STD>(P, A, l.z, none, frec, q);
            settle2(q);
        }
    } else {
        for (int k = 0; k < (nff & ~3); k += 4) {
            const uint4 l = list_quad_stream(ff, k, nf, s);
            FluidSums q;
            ff_pair32<ND, STD>(P, ta, va, p_a, rho_a, ia, drho_a, l.x, frec, q);
            ff_pair32<ND, STD>(P, ta, va, p_a, rho_a, ia, drho_a, l.y, frec, q);
            ff_pair32<ND, STD>(P, ta, va, p_a, rho_a, ia, drho_a, l.z, frec, q);
            ff_pair32<ND, STD>(P, ta, va, p_a, rho_a, ia, drho_a, l.w, frec, q);
            settle(q);
        }
        if (nff & 3) {  // the open quad: entries beyond the count are not part of the list
            const int k = nff & ~3, m = nff & 3;
            const uint4 l = list_quad_stream(ff, k, nf, s);
            FluidSums q;
            ff_pair32<ND, STD>(P, ta, va, p_a, rho_a, ia, drho_a, l.x, frec, q);
            if (m > 1) ff_pair32<ND, STD>(P, ta, va, p_a, rho_a, ia, drho_a, l.y, frec, q);
            if (m > 2) ff_pair32<ND, STD>(P, ta, va, p_a, rho_a, ia, drho_a, l.z, frec, q);
            settle(q);
        }
    }
    // the wall neighbours continue the same compensated sums
    const int nfw = fwc[s];
    for (int k = 0; k < (nfw & ~3); k += 4) {
        const uint4 l = list_quad_stream(fw, k, nf, s);
        FluidSums q;
        fw_pair32<ND>(P, ta, va, p_a, rho_a, ia, l.x, wtest[l.x & kSlotMask], wpres, q);
        fw_pair32<ND>(P, ta, va, p_a, rho_a, ia, l.y, wtest[l.y & kSlotMask], wpres, q);
        fw_pair32<ND>(P, ta, va, p_a, rho_a, ia, l.z, wtest[l.z & kSlotMask], wpres, q);
        fw_pair32<ND>(P, ta, va, p_a, rho_a, ia, l.w, wtest[l.w & kSlotMask], wpres, q);
        settle(q);
    }
    if (nfw & 3) {
        const int k = nfw & ~3, m = nfw & 3;
        const uint4 l = list_quad_stream(fw, k, nf, s);
        FluidSums q;
        fw_pair32<ND>(P, ta, va, p_a, rho_a, ia, l.x, wtest[l.x & kSlotMask], wpres, q);
        if (m > 1)
            fw_pair32<ND>(P, ta, va, p_a, rho_a, ia, l.y, wtest[l.y & kSlotMask], wpres, q);
        if (m > 2)
            fw_pair32<ND>(P, ta, va, p_a, rho_a, ia, l.z, wtest[l.z & kSlotMask], wpres, q);
        settle(q);
    }

    pair32_finish<ND, INTEGRATE>(U, s, va, drho_a, a0, a1, a2, ar, gate);
}

template <int ND, bool INTEGRATE, bool STD>
__global__ void __launch_bounds__(256, kPackedPairs<ND> ? 4 : 5) k_pair32(Phys32 P, int nf,
                                                const float4* __restrict__ frec,
                                                const unsigned* __restrict__ ff,
                                                const int* __restrict__ ffc,
                                                const unsigned* __restrict__ fw,
                                                const int* __restrict__ fwc,
                                                const float4* __restrict__ wtest,
                                                const float* __restrict__ wpres,
                                                unsigned* __restrict__ gate, Update32 U) {
    pair32_slot<ND, INTEGRATE, STD>(P, blockIdx.x * blockDim.x + threadIdx.x, nf, frec, ff,
                                    ffc, fw, fwc, wtest, wpres,
                                    gate, U);
}

// Batched persistent pair pass: one launch advances the pair stage of every member of a batch.
// The launch keeps about as many blocks as fit on the GPU; each block takes work items -- a tile
// of kBatchTile consecutive slots of one member, the largest member's tiles first -- from a
// counter in global memory (atomicAdd) until none is left, and runs the list pass on them.
template <int ND, bool STD>
__global__ void __launch_bounds__(kBatchTile, kPackedPairs<ND> ? 4 : 5) k_batch_pair32(const __grid_constant__ Pair32Batch B,
                                                                 unsigned* __restrict__ counter) {
    __shared__ int item;
    for (;;) {
        __syncthreads();  // every thread has read the previous item
        if (threadIdx.x == 0) item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = item;
        if (it >= B.tile0[B.n]) return;
        int m = 0;
        while (m + 1 < B.n && it >= B.tile0[m + 1]) ++m;
        const Pair32Member& M = B.m[m];
        const int s = (it - B.tile0[m]) * kBatchTile + threadIdx.x;
        pair32_slot<ND, true, STD>(M.P, s, M.nf, M.frec, M.ff, M.ffc,
                                   M.fw, M.fwc, M.wtest, M.wpres, M.gate, M.U);
    }
}

// ------------------------------------------------------------------------------------------
// Tiled pair pass (TP_PAIR_TILED): no neighbour lists.  Every warp enumerates the candidate
// cells of its 32 fluid slots directly from the cell list -- lanes grouped by their (cy, cz)
// row, the group's lanes bounded by a box, each neighbouring row's contiguous slot range
// streamed 32 records at a time (the enumeration of the list builder, tp_lists.cuh) -- and
// stages the records that pass the box test in shared memory with coalesced 16-byte loads:
// test record (x taken relative to the group's first cell), velocity record and pressure.  Each
// lane then tests every staged record against its own position (a broadcast shared load per
// record) into a 32-bit accept mask, and evaluates its accepted pairs from shared memory, one
// mask bit at a time, with the same pair terms as the list pass.  A quad of staged records
// feeds one blocked-Kahan partial as in the list pass (here: one partial per staged chunk).
// The reach (one or two cells towards a face, radius 2h (1 + skin) from the reference cell)
// covers every particle within 2h until the displacement gate reopens, exactly as for the
// lists; pairs are decided with |x_a - x_b|^2 <= (2h)^2 at use time.
// ------------------------------------------------------------------------------------------
struct TileStage {
    float4 t[32];  // {X relative to the group's first cell, oy, oz, rho - rho0 | m/rho (wall)}
    float4 v[32];  // fluid: {v, m / rho}
    float p[32];   // pressure
};

template <int ND, bool WALL, bool STD>
__device__ __forceinline__ void tile_sources(const Phys32& P, const GridDesc& g, float cs,
                                             float m, float r2list, bool active, const int c[3],
                                             float4 oa, float4 va, float p_a, float rho_a,
                                             float ia, float drho_a,
                                             const int* __restrict__ start,
                                             const int* __restrict__ skey,
                                             const float4* __restrict__ test,
                                             const float4* __restrict__ vel,
                                             const float* __restrict__ pres, TileStage& st,
                                             Kahan& a0, Kahan& a1, Kahan& a2, Kahan& ar) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int xl = reach_lo(oa.x, m), xh = reach_hi(oa.x, cs, m);
    const int yl = reach_lo(oa.y, m), yh = reach_hi(oa.y, cs, m);
    const int zl = (ND == 3) ? reach_lo(oa.z, m) : 0, zh = (ND == 3) ? reach_hi(oa.z, cs, m) : 0;
    const int yz = active ? (c[1] + g.n[1] * c[2]) : -1;
    const float margin = 1e-3f * cs;
    const float rbox = sqrtf(r2list) * 1.0001f + margin;
    const float r2box = rbox * rbox;
    unsigned todo = __ballot_sync(FULL, active);
    while (todo) {
        const int leader = __ffs(todo) - 1;
        const int yz0 = __shfl_sync(FULL, yz, leader);
        const int cx0 = __shfl_sync(FULL, c[0], leader);
        const bool ing = active && (yz == yz0);
        const unsigned grp = __ballot_sync(FULL, ing);
        todo &= ~grp;
        const int cy = yz0 % g.n[1], cz = yz0 / g.n[1];
        const float xlane = fmaf((float)(c[0] - cx0), cs, oa.x);
        const float ax = fmaxf(xlane, 0.0f);
        const float ay = fmaxf(oa.y, 0.0f), az = fmaxf(oa.z, 0.0f);
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
                if (fmaf(ey, ey, ez * ez) > r2box) continue;
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
                const float sy = fmaf(-(float)dy, cs, oa.y);
                const float sz = fmaf(-(float)dz, cs, oa.z);
                const float ryz = fmaf(ey, ey, ez * ez);
                for (int base = lo; base < hi; base += 32) {
                    const int j = base + lane;
                    bool rel = false;
                    float4 cb = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (j < hi) {
                        cb = test[j];
                        const int cxb = skey[j] - rb;
                        const float X = fmaf((float)(cxb - cx0), cs, cb.x);
                        cb.x = X;
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
                    const unsigned hits = __ballot_sync(FULL, rel);
                    if (rel) {
                        const int pos = __popc(hits & ((1u << lane) - 1u));
                        st.t[pos] = cb;
                        if (!WALL) st.v[pos] = vel[j];
                        st.p[pos] = pres[j];
                    }
                    __syncwarp();
                    const int nrel = __popc(hits);
                    // test phase: every lane against every staged record (broadcast loads)
                    unsigned acc = 0u;
                    if (ing) {
                        for (int i = 0; i < nrel; ++i) {
                            const float4 cbi = st.t[i];
                            const float pdx = xlane - cbi.x;
                            const float pdy = sy - cbi.y;
                            float d2 = fmaf(pdy, pdy, pdx * pdx);
                            if (ND == 3) {
                                const float pdz = sz - cbi.z;
                                d2 = fmaf(pdz, pdz, d2);
                            }
                            acc |= (d2 <= P.sr2 && d2 >= P.az2) ? (1u << i) : 0u;
                        }
                    }
                    // pair phase: the lane's accepted records, one mask bit at a time
                    if (acc) {
                        FluidSums q;
                        do {
                            const int i = __ffs(acc) - 1;
                            acc &= acc - 1u;
                            const float4 cbi = st.t[i];
                            const float pd0 = xlane - cbi.x, pd1 = sy - cbi.y;
                            const float pd2 = (ND == 3) ? sz - cbi.z : 0.0f;
                            float d2 = fmaf(pd1, pd1, pd0 * pd0);
                            if (ND == 3) d2 = fmaf(pd2, pd2, d2);
                            if (WALL)
                                fw_terms32<ND>(P, va, p_a, rho_a, ia, pd0, pd1, pd2, d2, cbi.w,
                                               st.p[i], q);
                            else
                                ff_terms32<ND, STD>(P, va, p_a, rho_a, ia, drho_a, pd0, pd1, pd2,
                                                    d2, cbi, st.v[i], st.p[i], q);
                        } while (acc);
                        a0.add(q.x);
                        a1.add(q.y);
                        if (ND == 3) a2.add(q.z);
                        ar.add(q.r);
                    }
                    __syncwarp();
                }
            }
        }
    }
}

template <int ND, bool INTEGRATE, bool STD>
__global__ void __launch_bounds__(256, 3) k_pair32_tiled(
    Phys32 P, GridDesc g, float m, float r2list, int nf, const int* __restrict__ fstart,
    const int* __restrict__ fskey, const float4* __restrict__ ftest,
    const float4* __restrict__ fvel, const float* __restrict__ fpres,
    const int* __restrict__ wstart, const int* __restrict__ wskey,
    const float4* __restrict__ wtest, const float* __restrict__ wpres, int nw,
    unsigned* __restrict__ gate, Update32 U) {
    __shared__ TileStage stage_all[8];
    TileStage& st = stage_all[threadIdx.x >> 5];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s < nf;
    const int si = active ? s : 0;
    const float4 ta = ftest[si];
    const float4 va = fvel[si];
    const float p_a = fpres[si];
    const float drho_a = ta.w;
    const float rho_a = P.rho0 + drho_a;
    const float ia = __frcp_rn(rho_a);
    int c[3];
    key_to_coords(fskey[si], g, c);
    Kahan a0, a1, a2, ar;
    tile_sources<ND, false, STD>(P, g, P.cs, m, r2list, active, c, ta, va, p_a, rho_a, ia,
                                 drho_a, fstart, fskey, ftest, fvel, fpres, st, a0, a1, a2, ar);
    if (nw > 0)
        tile_sources<ND, true, STD>(P, g, P.cs, m, r2list, active, c, ta, va, p_a, rho_a, ia,
                                    drho_a, wstart, wskey, wtest, nullptr, wpres, st, a0, a1, a2,
                                    ar);
    if (!active) return;
    pair32_finish<ND, INTEGRATE>(U, s, va, drho_a, a0, a1, a2, ar, gate);
}
// ------------------------------------------------------------------------------------------
// Host launchers
// ------------------------------------------------------------------------------------------
namespace {
inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }
}

void fp32_pack(tp_handle* h, const double* u, const double* v, const double* m,
               const PhysState* src, PhysState* dst, const unsigned* gate, bool skip_in_place) {
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
        const bool dense = h->pair_mode == TP_PAIR_TILED;
        pk.test = dense ? h->f_test : nullptr;
        pk.vel = dense ? (float4*)h->f_vel : nullptr;
        pk.pres = dense ? (float*)h->f_aux : nullptr;
        pk.rec = (float4*)h->f_rec;
        pk.skip_in_place = skip_in_place;
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
            (const float4*)h->f_rec);
    else
        k_adami32<3><<<nblk(nw, h->pair_block), h->pair_block, 0, h->stream>>>(
            h->phys32, nw, h->w_test, h->l_wf, h->c_wf, (float4*)h->w_state, h->w_p32, h->w_vol,
            (const float4*)h->f_rec);
}

template <int ND, bool INTEG>
static void launch_pair32(tp_handle* h, unsigned* gate, const Update32& U) {
    const int nf = (int)h->cfg.n_fluid;
    const Phys32& P = h->phys32;
    const bool std_cfg = P.visc && P.beta == 0.0f && P.diff;
    auto run = [&](auto stdc) {
        if (h->pair_mode == TP_PAIR_TILED) {
            // candidate enumeration of the list builder at radius 2h (1 + skin)
            const double r = 2.0 * h->cfg.smoothing_length * (1.0 + h->skin);
            const float r2list = (float)(r * r * (1.0 + 1e-5));
            const float m = (float)(r - h->grid.cs + 1e-5 * h->grid.cs);
            k_pair32_tiled<ND, INTEG, decltype(stdc)::value><<<nblk(nf, 256), 256, 0,
                                                              h->stream>>>(
                P, h->grid, m, r2list, nf, h->f_start, h->f_skey, h->f_test,
                (const float4*)h->f_vel, (const float*)h->f_aux, h->w_start, h->w_skey,
                h->w_test, h->w_p32, (int)h->cfg.n_wall, gate, U);
            return;
        }
        k_pair32<ND, INTEG, decltype(stdc)::value><<<nblk(nf, h->pair_block), h->pair_block, 0,
                                                     h->stream>>>(
            P, nf, (const float4*)h->f_rec, h->l_ff, h->c_ff, h->l_fw, h->c_fw, h->w_test,
            h->w_p32, gate, U);
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
                     double dt, int first, Pair32Member* desc, bool fuse_next) {
    if (h->cfg.n_fluid == 0 && !desc) return;
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
    if (fuse_next) {  // the next stage's records into the other buffer (swapped after the stage)
        U.rec_next = (float4*)h->f_rec2;
        U.skey = h->f_skey;
        U.grid = h->grid;
        U.cs32 = (double)(float)h->grid.cs;
        U.rho0 = h->phys32.rho0;
        U.id_in = st.id;          // the next stage's source: this stage's destination
        U.id_out = src.id;        // the next stage's destination
        U.m_in = (const float*)st.m;
        U.m_out = (float*)src.m;
    }
    if (desc) {  // the batched persistent pass launches it (fp32_batch_pair)
        Pair32Member& M = *desc;
        M.P = h->phys32;
        M.nf = (int)h->cfg.n_fluid;
        M.frec = (const float4*)h->f_rec;
        M.ff = h->l_ff;
        M.ffc = h->c_ff;
        M.fw = h->l_fw;
        M.fwc = h->c_fw;
        M.wtest = h->w_test;
        M.wpres = h->w_p32;
        M.gate = h->gate;
        M.U = U;
        return;
    }
    if (h->cfg.ndims == 2)
        launch_pair32<2, true>(h, h->gate, U);
    else
        launch_pair32<3, true>(h, h->gate, U);
}

// p of every fluid slot to caller order (tp_fluid_pressure): the Cole EOS of the record's
// rho - rho0, the value the pack and the pair pass use.
__global__ void k_scatter_pressure32(Phys32 P, const float4* __restrict__ rec,
                                     const int* __restrict__ perm, double* __restrict__ p, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) p[perm[s]] = (double)eos32(rec[2 * (size_t)s].w, P, P.fluid_clip);
}

void fp32_scatter_pressure(tp_handle* h, const int* ids, double* p_fluid) {
    const int nf = (int)h->cfg.n_fluid;
    k_scatter_pressure32<<<nblk(nf, 256), 256, 0, h->stream>>>(
        h->phys32, (const float4*)h->f_rec, ids, p_fluid, nf);
}

bool fp32_batch_pair_std(const Phys32& P) { return P.visc && P.beta == 0.0f && P.diff; }

tp_status fp32_batch_pair(const Pair32Batch& B, int nd, bool std_cfg, unsigned* counter,
                          cudaStream_t stream) {
    int per_sm = 0, sms = 0, dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto run = [&](auto ndc, auto stdc) {
        constexpr int ND = decltype(ndc)::value;
        constexpr bool S = decltype(stdc)::value;
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_pair32<ND, S>,
                                                              kBatchTile, 0);
        const int blocks = std::max(1, std::min(B.tile0[B.n], std::max(per_sm, 1) * sms));
        if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, sizeof(unsigned), stream);
        if (e == cudaSuccess) k_batch_pair32<ND, S><<<blocks, kBatchTile, 0, stream>>>(B, counter);
    };
    if (nd == 2) {
        if (std_cfg) run(std::integral_constant<int, 2>{}, std::true_type{});
        else run(std::integral_constant<int, 2>{}, std::false_type{});
    } else {
        if (std_cfg) run(std::integral_constant<int, 3>{}, std::true_type{});
        else run(std::integral_constant<int, 3>{}, std::false_type{});
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? TP_OK : TP_ERR_CUDA;
}

}  // namespace tp
