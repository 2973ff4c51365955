// tp_internal.cuh — shared device-side definitions of the sm_103a WCSPH library.
//
// Data layout in HBM (all particle arrays are cell-sorted "slots" unless noted; o = offset of
// the particle inside its reference cell in FP32 metres, cx = its x cell index):
//   fluid records, written by the pack pass of every right-hand side:
//     both forms: ftest[s] = float4 {ox, oy, oz, cx} (FP64) / {ox, oy, oz, rho - rho0} (FP32)
//     FP64 form:  fpos[s] = double4_32a {x, y, z, p}   fvel[s] = double4_32a {vx, vy, vz, rho}
//                 faux[s] = double4_32a {p S, S, p_off + p - rho g.x, 2 m alpha c h sg_c} with
//                 S = sg_c m / rho (gather pair mode; the symmetric mode keeps {m, m/rho, 1/rho,
//                 2 m alpha c h})
//     FP32 form:  fvel[s] = float4 {vx, vy, vz, m / rho}   faux[s] = float p (written for the
//                 tiled pair pass; the list pass reads frec[2s..2s+1] = {test, vel})
//   wall records, sorted once (walls are static), the state rewritten by the Adami pass:
//     wpos[s] = double4_32a {x, y, z, m}, wtest[s] = float4 {ox, oy, oz, cx} (FP32 form: the
//     fourth slot is m / rho of the last Adami pass)
//     FP64:  wstate[s] = double4_32a {p, rho, p S, S}  (symmetric mode: {p, rho, 1/rho, m/rho})
//     FP32:  wstate[s] = float4 {p, rho - rho0, m, m / rho} and a dense float pressure array
//   cell list: start[c] = first slot of cell c (ncells + 1 entries), cells linearised x fastest,
//   so the three cells (cx-1, cx, cx+1) of one (cy, cz) row are one contiguous slot range;
//   neighbour lists in the chunked layout of tp_lists.cuh.
// In 2D the z components are unused.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tp_wcsph.h"

#define TP_ERRBIT_OUT_OF_GRID 1
#define TP_ERRBIT_NONFINITE 2

namespace tp {

// Padded cell grid: cell coordinate along d is floor(x_d / cs) - cmin[d]; valid particle cells
// are 1..n[d]-2 (one padding layer each side), so every 3^d neighbourhood is inside the grid.
struct GridDesc {
    int nd;
    double cs;
    int cmin[3];
    int n[3];
    int ncells;
    // optional (device): the cell origins (cmin + c) * cs32 of the FP32 cell size per axis, axis d
    // from org + n[0] (d > 0) + n[1] (d > 1), so that the test records take no FP64 product
    const double* org = nullptr;
};

// Physical parameters, precomputed on the host in FP64 following the reference expressions.
struct Phys {
    int nd;
    double h;          // smoothing length
    double h_inv;      // 1 / h
    double sr2;        // (2h)^2, neighbour criterion d2 <= sr2
    double two_h;      // compact support 2h (kernel() cut, strict <)
    double almostzero; // sqrt(eps((2h)^2)), rhs.jl:27-28
    double az2;        // eps((2h)^2): the zero-distance skip on d^2
    double wc2_norm;   // WendlandC2 normalisation sigma_d * h_inv^d (smoothing_kernels.jl:450-455)
    double wc2_dnorm;  // -5 * wc2_norm (kernel_deriv_div_r_unsafe prefactor)
    double hi2;        // h_inv * h_inv
    double rho0, c, gamma, p_bg, B, inv_gamma;
    int gamma_int;     // the exponent when it is an integer in [1, 16], else 0
    int fluid_clip, wall_clip;
    int visc;
    double alpha, beta, eps_visc;
    double visc_h;     // (h + h) / 2
    double visc_eps_h2;  // eps * (visc_h * visc_h)
    double visc_mac;   // alpha * c  (used as ((m_b*alpha)*c) in FP64 order)
    int diff;
    double delta;
    double diff_coef;  // (delta * ((h + h) / 2)) * c
    double g[3];
    double p_off;
    // derived constants of the FP64 pair kernels
    double sg_c;       // wc2_dnorm * hi2: grad W = sg_c (1 - q/2)^3 x_ab
    double half_hinv;  // 0.5 * h_inv: 1 - q/2 = 1 - r * half_hinv
    double visc_k;     // alpha * c * visc_h (Monaghan with beta = 0)
    double visc_k2;    // 2 * visc_k (per-particle 2 m alpha c h of the pack)
    double visc_k2s;   // visc_k2 * sg_c (gather-mode record: 2 m alpha c h sg_c)
    double alpha_c;    // alpha * c
    double diff2;      // 2 * diff_coef
};

// FP32 copies of the constants used by the precision form.
struct Phys32 {
    float cs;          // cell size rounded to FP32 (offsets are taken against it)
    float h_inv, sr2, two_h, almostzero, wc2_norm, wc2_dnorm, hi2;
    float rho0, B, gamma, inv_gamma, p_bg;
    int fluid_clip, wall_clip, visc, diff;
    float beta, visc_h, visc_eps_h2, visc_ac, diff_coef;
    float g[3];
    float p_off;
    // derived constants of the FP32 pair kernel (see the FP64 ones)
    float sg_c, half_hinv, visc_k, diff2, az2;
    // Cole EOS with the exponent 7: evaluated as a polynomial in (rho - rho0) / rho0
    int gamma7;
    float inv_rho0;
};

// Stage update of the FP32 pair pass (kick! output or fused CK2N54 register update).
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
    // optional: the next stage's 32-byte records of the new state (rec_next[2s], [2s + 1]) as the
    // next stage's pack would write them without a rebuild, with the slot's reference cell skey[s],
    // and the id / mass copy into the destination state
    float4* rec_next;
    const int* skey;
    GridDesc grid;
    double cs32;
    float rho0;
    const int* id_in;
    int* id_out;
    const float* m_in;
    float* m_out;
};

// One member of the batched persistent FP32 pair pass: everything its list pass reads.
struct Pair32Member {
    Phys32 P;
    int nf;
    const float4* frec;
    const unsigned* ff;
    const int* ffc;
    const unsigned* fw;
    const int* fwc;
    const float4* wtest;
    const float* wpres;
    unsigned* gate;
    Update32 U;
};

constexpr int kBatchMaxMembers = 6;
constexpr int kBatchTile = 256;  // slots per work item of the persistent pass (one per thread)

// Kernel parameter of the persistent pass (passed by value, read in place as __grid_constant__).
struct Pair32Batch {
    Pair32Member m[kBatchMaxMembers];
    int tile0[kBatchMaxMembers + 1];  // first work item of each member; tile0[n] = total
    int n;
};

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Cell coordinates of x (FP64).  Returns an error bit (0 = inside the inner grid); the coordinate
// is clamped into the inner grid so that later passes never index outside the arrays.
template <int ND>
__device__ __forceinline__ int cell_coords(const double* x, const GridDesc& g, int c[3]) {
    int err = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d < ND) {
            double q = __ddiv_rn(x[d], g.cs);
            double gd = floor(q) - (double)g.cmin[d];
            if (!(gd >= 1.0 && gd <= (double)(g.n[d] - 2))) {
                err |= (x[d] != x[d] || isinf(x[d])) ? TP_ERRBIT_NONFINITE : TP_ERRBIT_OUT_OF_GRID;
                gd = (gd != gd) ? 1.0 : fmin(fmax(gd, 1.0), (double)(g.n[d] - 2));
            }
            c[d] = (int)gd;
        } else {
            c[d] = 0;
        }
    }
    return err;
}

__device__ __forceinline__ int cell_key(const int c[3], const GridDesc& g) {
    return c[0] + g.n[0] * (c[1] + g.n[1] * c[2]);
}

__device__ __forceinline__ void key_to_coords(int key, const GridDesc& g, int c[3]) {
    c[0] = key % g.n[0];
    int r = key / g.n[0];
    c[1] = r % g.n[1];
    c[2] = r / g.n[1];
}

// x^n for a small positive integer n by squaring (x^7: four multiplications, a few ulp of the
// correctly rounded power).  FP64 runs at 1/64 of the FP32 rate on this GPU, and pow's
// logarithm and exponential cost tens of FP64 instructions per call.
__device__ __forceinline__ double ipow(double x, int n) {
    double r = 1.0, b = x;
    while (n) {
        if (n & 1) r *= b;
        n >>= 1;
        if (n) b *= b;
    }
    return r;
}

// StateEquationCole pressure (state_equations.jl:117-129), FP64; an integer exponent (the usual
// 7) by repeated multiplication.
__device__ __forceinline__ double eos_pressure(double rho, const Phys& P, int clip) {
    const double x = rho / P.rho0;
    const double xg = P.gamma_int ? ipow(x, P.gamma_int) : pow(x, P.gamma);
    double p = P.B * (xg - 1.0) + P.p_bg;
    if (clip) p = (p != p || p > 0.0) ? p : 0.0;
    return p;
}

// a^(1/n) for a > 0 and a small positive integer n: an FP32 seed and two Newton steps
// y <- y + y (a / y^n - 1) / n in FP64 (the error squares from 1e-7 to rounding level, a few ulp
// of the correctly rounded root), a third of FP64 pow's cost; a = y^n exactly stays exact.
__device__ __forceinline__ double iroot(double a, int n) {
    double y = (double)powf((float)a, 1.0f / (float)n);
#pragma unroll
    for (int it = 0; it < 2; ++it) y = fma(y, (a / ipow(y, n) - 1.0) / (double)n, y);
    return y;
}

// inverse_state_equation (state_equations.jl:131-139), FP64; an integer exponent by iroot.
__device__ __forceinline__ double eos_inverse(double p, const Phys& P) {
    double tmp = (p - P.p_bg) / P.B + 1.0;
    return P.rho0 * (P.gamma_int && tmp > 0.0 ? iroot(tmp, P.gamma_int) : pow(tmp, P.inv_gamma));
}

}  // namespace tp
