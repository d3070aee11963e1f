// sm_103a kernels of the spectral-element time step, templated on the
// polynomial degree N (lpd), the wavefield precision T, the number of
// standard linear solids and anisotropy. One translation unit per degree
// instantiates them (kern_lpd<N>.cu).
//
// Per step (src/evolution.f90:87-444 followed by the driver's add/record,
// src/ses3d-nt.F90:240-250):
//   k_element  one thread per element-local GLL point, EPB elements per block:
//              gather v of the element's points from the unique-point array
//              into shared memory; nine line contractions for the velocity
//              gradient (:130-159); spherical completion and symmetrisation
//              (:165-173, :206-208); stress rate and integration (:287-311),
//              or the standard-linear-solid form with its memory variables
//              (:216-284, :415-442); taper of the stored stress (:404-409);
//              the weak divergence (:332-367) as nine transposed line
//              contractions over metric-weighted stresses in shared memory;
//              assembly by atomic adds into the unique-point force
//              (replaces :372-388 and src/communicate_fields.F90:48-247).
//   k_sources  the moment-tensor / single-force slabs (channel_mod.f90:859-1095)
//              pushed through the same weak divergence, added to the force.
//   k_node     one thread per unique point: v += dt * F / M, taper
//              (:393-402), force reset for the next step.
//   k_receivers one warp per receiver: Lagrange interpolation of v
//              (channel_mod.f90:505-592).
// Variants of the element kernel: element_tc.cuh (tcgen05 contractions),
// element_tma.cuh (persistent, state moved by bulk copies); channels.cuh holds
// the receiver-channel and snapshot-field kernels.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "sesnt.h"
#include "sesnt_internal.h"

namespace sesnt {

// Launch shape of the element kernel, chosen by measurement on GB300 (config-2
// workload, lpd 4, 3 SLS): one element per 128-thread block with registers
// sized for 8 resident blocks beat 2 or 4 elements per block by 7-10%.
#ifndef SESNT_EPB_LPD4
#define SESNT_EPB_LPD4 1
#endif
#ifndef SESNT_MINB_256
#define SESNT_MINB_256 4
#endif
// lpd 6 (352-thread blocks): registers sized for 3 resident blocks measured
// 15% faster than 2 (config 3, 96x96x48) and than 4 (spills).
#ifndef SESNT_MINB_384
#define SESNT_MINB_384 3
#endif
// Where k_element loads the SLS memory variables: with the other loads at
// the start (0) or right after the barrier that stages the velocities,
// before the line contractions and any store (1).
// -1 picks by degree: late up to degree 5, early for 6 and 7. Measured on
// 3-SLS FP32 grids of 6-12 M points: late is 4.3/1.2/3.9/5.0% faster for
// degrees 2/3/4/5 and 1.4/2.4% slower for 6/7; FP64 (degree 4) unchanged.
#ifndef SESNT_LATE_MEM
#define SESNT_LATE_MEM -1
#endif
// Resident blocks the paired-simulation elastic kernel is sized for (FP32):
// 8 (64 registers, no spills) measured 1% faster than 6 and 5% faster than 4.
#ifndef SESNT_MINB_PAIR
#define SESNT_MINB_PAIR 8
#endif

template <int N>
struct ElemCfg {
    static constexpr int P = N + 1;
    static constexpr int NP = P * P * P;
    // elements per block: enough points to fill whole warps with little waste
    static constexpr int EPB = N == 4 ? SESNT_EPB_LPD4 : (NP <= 32 ? 8 : (NP <= 64 ? 2 : (NP <= 128 ? 2 : 1)));
    static constexpr int NT = ((EPB * NP + 31) / 32) * 32;
    // resident blocks per SM the register allocation is sized for
    static constexpr int MINB = NT <= 128 ? 2 * SESNT_MINB_256
                              : (NT <= 256 ? SESNT_MINB_256 : (NT <= 384 ? SESNT_MINB_384 : (NT <= 512 ? 2 : 1)));
    // the same for the paired-simulation elastic kernel (two points' state per thread)
    static constexpr int MINB_PAIR = NT <= 128 ? SESNT_MINB_PAIR : (NT <= 256 ? 3 : (NT <= 384 ? 2 : 1));
};

// Bounds-check builds (-DSESNT_BOUNDS_CHECK): a global index outside its
// buffer sets bit 2 of the error word and the access is skipped; no device
// assert, no trap. In normal builds the check compiles away.
__device__ __forceinline__ bool in_range(size_t idx, size_t n, int *err) {
#ifdef SESNT_BOUNDS_CHECK
    if (idx < n) return true;
    atomicOr(err, 2);
    return false;
#else
    (void)idx;
    (void)n;
    (void)err;
    return true;
#endif
}

// Assembly of one element-local point's force into the unique-point force of
// simulation s (replaces src/evolution.f90:372-388 and
// src/communicate_fields.F90:48-247): FP32 atomic adds into F, or with
// SESNT_FLAG_FORCE64 FP64 atomic adds into F64. The assembled force of a
// smooth field is a small difference of large per-element contributions;
// summed in FP64 it loses no digits to that cancellation.
template <typename T>
__device__ __forceinline__ void add_force(const StepArgs<T> &a, int s, size_t u, T fx, T fy, T fz) {
    const size_t nuni = (size_t)a.nuni;
    if (a.F64) {
        double *F = a.F64 + (size_t)s * 3 * nuni;
        atomicAdd(F + u, (double)fx);
        atomicAdd(F + nuni + u, (double)fy);
        atomicAdd(F + 2 * nuni + u, (double)fz);
    } else {
        T *F = a.F + (size_t)s * 3 * nuni;
        atomicAdd(F + u, fx);
        atomicAdd(F + nuni + u, fy);
        atomicAdd(F + 2 * nuni + u, fz);
    }
}

// Evict-first hints: measured faster on the stores only (loads without the
// hint keep the next blocks' shared velocity lines warm).
#ifndef SESNT_HINT_LOADS
#define SESNT_HINT_LOADS 0
#endif
#ifndef SESNT_HINT_STORES
#define SESNT_HINT_STORES 1
#endif
// Streamed element-local data (stress, memory variables, material) with or
// without the evict-first cache hint.
template <typename T>
__device__ __forceinline__ T ld_stream(const T *p) {
#if SESNT_HINT_LOADS
    return __ldcs(p);
#else
    return *p;
#endif
}
template <typename T>
__device__ __forceinline__ void st_stream(T *p, T v) {
#if SESNT_HINT_STORES
    __stcs(p, v);
#else
    *p = v;
#endif
}

// Taper from the three damping profiles (src/geometric_paras.f90:308-316):
// corner normalisation, then exp(-0.1*prof^2).
template <typename T>
__device__ __forceinline__ T taper_value(T px, T py, T pz, T inv_alpha) {
    const T prof = px + py + pz;
    if (prof == T(0)) return T(1);
    const T s = T(2) / (T(1) + prof * inv_alpha);
    const T p2 = (px + py + pz) * s;
    return exp(-(T(0.1) * (p2 * p2)));
}

// Per-point pieces of the element kernels. From the point's velocity
// gradient and its stress, memory variables and material: spherical
// completion, stress rate (elastic or standard linear solids, optional
// A,B,C), integration, taper of the stored stress, memory-variable update,
// and the metric-weighted stresses of the weak divergence written to the flux
// slab `my` (9 x NP).
// Raw velocity gradient at point (i,j,k): the nine line contractions of the
// velocity slab with the scaled derivative tables (src/evolution.f90:130-159).
// e[d*3 + c] = d-direction derivative of component c (d, c in x, y, z).
template <int N, typename T>
__device__ __forceinline__ void strain_contract(const T *sD, const T *svx, const T *svy, const T *svz, int i, int j,
                                                int k, T (&e)[9]) {
    constexpr int P = N + 1;
    const T *Dx = sD, *Dy = sD + P * P, *Dz = sD + 2 * P * P;
#pragma unroll
    for (int c = 0; c < 9; ++c) e[c] = 0;
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const int px_ = q + P * (j + P * k);
        const int py_ = i + P * (q + P * k);
        const int pz_ = i + P * (j + P * q);
        const T dx = Dx[q * P + i], dy = Dy[q * P + j], dz = Dz[q * P + k];
        e[0] += svx[px_] * dx;
        e[1] += svy[px_] * dx;
        e[2] += svz[px_] * dx;
        e[3] += svx[py_] * dy;
        e[4] += svy[py_] * dy;
        e[5] += svz[py_] * dy;
        e[6] += svx[pz_] * dz;
        e[7] += svy[pz_] * dz;
        e[8] += svz[pz_] * dz;
    }
}

// Spherical completion of the raw velocity gradient e[9] (layout of
// strain_contract) at point (i, ., k) of element (ex, ., ez)
// (src/evolution.f90:165-173; theta = x, phi = y, r = z). Divisions by r and
// r*sin(theta) are products with tabulated reciprocals. Output g[9] in the
// order kDu* (xx yy zz xy yx xz zx yz zy), not yet symmetrised.
// The completion from the point's metric values: ir = 1/r, ct = cot(theta),
// irs = 1/(r sin(theta)).
template <typename T>
__device__ __forceinline__ void complete_gradient_m(const T (&e)[9], T vx, T vy, T vz, T ir, T ct, T irs,
                                                    T (&g)[9]) {
    T exx = e[0], exy = e[1], exz = e[2], eyx = e[3], eyy = e[4], eyz = e[5], ezx = e[6], ezy = e[7], ezz = e[8];
    ezz = -ezz;
    eyy = eyy * irs + (vz + vx * ct) * ir;
    exx = (vz + exx) * ir;
    ezx = -ezx;
    exz = (exz - vx) * ir;
    ezy = -ezy;
    eyz = -vy * ir + eyz * irs;
    exy = exy * ir;
    eyx = -(vy * ct) * ir + eyx * irs;
    g[kDuXX] = exx; g[kDuYY] = eyy; g[kDuZZ] = ezz;
    g[kDuXY] = exy; g[kDuYX] = eyx; g[kDuXZ] = exz;
    g[kDuZX] = ezx; g[kDuYZ] = eyz; g[kDuZY] = ezy;
}

template <int N, typename T>
__device__ __forceinline__ void complete_gradient(const StepArgs<T> &a, const T (&e)[9], T vx, T vy, T vz, int i,
                                                  int k, int ex, int ez, T (&g)[9]) {
    constexpr int P = N + 1;
    const T ir = a.inv_r[ez * P + k];
    const T ct = a.cot_t[ex * P + i];
    const T irs = ir * a.inv_sin[ex * P + i];
    complete_gradient_m<T>(e, vx, vy, vz, ir, ct, irs, g);
}

// Metric values of one point that a caller has already loaded (the column
// kernels hold the column-invariant ones in registers): 1/r, cot(theta),
// 1/sin(theta), r, sin(theta), the three taper profiles, w_i * w_j and w_k.
template <typename T>
struct PointMetric {
    T ir, ct, isn, rr, st, px, py, pz, wij, wk;
};

// Stress rates from the symmetrised strain rates (src/evolution.f90:287-296),
// or the standard-linear-solid form with the memory variables m
// (:216-284, the commented branch, with the Mxy/Mxz/Myz sums fixed), plus
// the anisotropic A, B, C terms.
template <typename T, int NSLS, bool ANISO>
__device__ __forceinline__ void stress_rates(T exx, T eyy, T ezz, T exy, T exz, T eyz, T lam, T mu, T tau, T cA,
                                             T cB, T cC, const T (&m)[6][NSLS > 0 ? NSLS : 1], T &rxx, T &ryy,
                                             T &rzz, T &rxy, T &rxz, T &ryz) {
    const T third = T(1) / T(3);
    const T two_mu = T(2) * mu;
    const T tr = exx + eyy + ezz;
    if constexpr (NSLS > 0) {
        const T mu_tau = (T(1) + tau) * mu;
        const T kappa = lam + two_mu * third;
        T sm[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            T acc = 0;
#pragma unroll
            for (int q = 0; q < NSLS; ++q) acc += m[c][q];
            sm[c] = acc;
        }
        const T tmt = T(2) * mu_tau;
        const T L = (kappa - tmt * third) * tr - two_mu * (sm[0] + sm[1] + sm[2]) * third;
        rxx = L + tmt * exx + two_mu * sm[0];
        ryy = L + tmt * eyy + two_mu * sm[1];
        rzz = L + tmt * ezz + two_mu * sm[2];
        rxy = tmt * exy + two_mu * sm[3];
        rxz = tmt * exz + two_mu * sm[4];
        ryz = tmt * eyz + two_mu * sm[5];
    } else {
        const T L = lam * tr;
        rxx = L + two_mu * exx;
        ryy = L + two_mu * eyy;
        rzz = L + two_mu * ezz;
        rxy = two_mu * exy;
        rxz = two_mu * exz;
        ryz = two_mu * eyz;
    }
    if constexpr (ANISO) {
        rxx += cC * ezz + cA * (eyy + exx);
        ryy += cC * ezz + cA * (eyy + exx);
        rzz += cC * (eyy + exx);
        rxz += T(2) * cB * exz;
        ryz += T(2) * cB * eyz;
    }
}

// The rest of one element-local point's step, from its raw velocity gradient
// e[9] (layout of strain_contract) and velocity, up to the stored stress:
// completion, stress rate, integration, the tapered stress and memory
// variables stored, and in sn[6] (xx xy xz yy yz zz) the integrated stress
// before the taper with gw[3] its metric weights for the weak divergence.
// DU: integrate this point's displacement gradient `du` (stride nloc); a
// compile-time switch, since even a skipped branch measured 1.5% on the
// step. SMEM: sig/mem point into shared memory (plain stores instead of
// streaming global stores).
// PM: the metric values come from *pm (PointMetric) instead of the tables.
// KS: compensated (Kahan) stress integration (SESNT_FLAG_KAHAN_STRESS): sigc
// points to the point's six compensation terms (global memory, stride cs),
// which carry the low-order part the FP32 stress loses at each step. The
// compensation is tapered with the stress and also takes up the rounding of
// the taper's product.
template <int N, typename T, int NSLS, bool ANISO, bool DU = false, bool SMEM = false, bool PM = false,
          bool KS = false>
__device__ __forceinline__ void point_stress(const StepArgs<T> &a, const T (&e)[9], T vx, T vy, T vz, int i, int j,
                                             int k, int ex, int ey, int ez, T lam, T mu, T tau, T cA, T cB, T cC,
                                             const T (&sg)[6], const T (&m)[6][NSLS > 0 ? NSLS : 1], T *sig, T *mem,
                                             size_t cs, size_t nloc, T *du, T (&sn)[6], T (&gw)[3],
                                             const PointMetric<T> *pm = nullptr, T *sigc = nullptr) {
    constexpr int P = N + 1;
    T g[9];
    if constexpr (PM) complete_gradient_m<T>(e, vx, vy, vz, pm->ir, pm->ct, pm->ir * pm->isn, g);
    else complete_gradient<N, T>(a, e, vx, vy, vz, i, k, ex, ez, g);
    T exx = g[kDuXX], eyy = g[kDuYY], ezz = g[kDuZZ], exy = g[kDuXY], eyx = g[kDuYX], exz = g[kDuXZ],
      ezx = g[kDuZX], eyz = g[kDuYZ], ezy = g[kDuZY];
    T rr, rs;
    if constexpr (PM) {
        rr = pm->rr;
        rs = rr * pm->st;
    } else {
        rr = a.r[ez * P + k];
        rs = rr * a.sin_t[ex * P + i];
    }
    if constexpr (DU) {
        // displacement gradient du += dt * (completed velocity gradient)
        // before the symmetrisation (src/evolution.f90:179-187)
#pragma unroll
        for (int c = 0; c < 9; ++c) du[c * nloc] = du[c * nloc] + a.dt * g[c];
    }
    exy = (exy + eyx) * T(0.5);
    exz = (exz + ezx) * T(0.5);
    eyz = (eyz + ezy) * T(0.5);

    T rxx, ryy, rzz, rxy, rxz, ryz;
    stress_rates<T, NSLS, ANISO>(exx, eyy, ezz, exy, exz, eyz, lam, mu, tau, cA, cB, cC, m, rxx, ryy, rzz, rxy, rxz,
                                 ryz);
    // integrate, taper the stored stress
    T sxx, sxy, sxz, syy, syz, szz, cn[6];
    if constexpr (KS) {
        // s + dt*r with the compensation c of the previous step: y = dt*r - c,
        // t = s + y, new compensation (t - s) - y
        const T r6[6] = {rxx, rxy, rxz, ryy, ryz, rzz};
        T o[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const T y = a.dt * r6[q] - ld_stream(sigc + q * cs);
            o[q] = sg[q] + y;
            cn[q] = (o[q] - sg[q]) - y;
        }
        sxx = o[0]; sxy = o[1]; sxz = o[2]; syy = o[3]; syz = o[4]; szz = o[5];
    } else {
        sxx = sg[0] + a.dt * rxx;
        sxy = sg[1] + a.dt * rxy;
        sxz = sg[2] + a.dt * rxz;
        syy = sg[3] + a.dt * ryy;
        syz = sg[4] + a.dt * ryz;
        szz = sg[5] + a.dt * rzz;
    }
    const T tp = PM ? taper_value(pm->px, pm->py, pm->pz, a.inv_alpha)
                    : taper_value(a.px[ex * P + i], a.py[ey * P + j], a.pz[ez * P + k], a.inv_alpha);
    auto put = [](T *q, T v) {
        if constexpr (SMEM) *q = v;
        else st_stream(q, v);
    };
    put(sig, sxx * tp);
    put(sig + cs, sxy * tp);
    put(sig + 2 * cs, sxz * tp);
    put(sig + 3 * cs, syy * tp);
    put(sig + 4 * cs, syz * tp);
    put(sig + 5 * cs, szz * tp);
    if constexpr (KS) {
        // the taper's product rounds too: with s' = t*tp as stored, the tapered
        // sum is s' - (c*tp + (s' - t*tp)), and fma gives t*tp - s' exactly
        const T o6[6] = {sxx, sxy, sxz, syy, syz, szz};
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const T stored = o6[q] * tp;
            st_stream(sigc + q * cs, cn[q] * tp - fma(o6[q], tp, -stored));
        }
    }
    if constexpr (NSLS > 0) {
        // memory variables after the update, driven by this step's rates:
        // M <- M - M*(dt/tau_p) - tau*dt/(n*tau_p)*e, the reference's form
        // (src/evolution.f90:415-442). Folding the decay into one factor
        // (1 - dt/tau_p) rounds that factor near 1 and biases the decay rate
        // of every step the same way: by 6.3e-4 of dt/tau_p for tau_p =
        // 1000 s and dt = 0.03 s. Kept apart, the rate dt/tau_p is rounded
        // to 2^-24 of itself.
        const T er[6] = {exx, eyy, ezz, exy, exz, eyz};
#pragma unroll
        for (int q = 0; q < NSLS; ++q) {
            const T drive = tau * a.mem_drive[q];
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const T mo = m[c][q];
                put(mem + (size_t)(c * NSLS + q) * cs, (mo - mo * a.mem_rate[q]) - drive * er[c]);
            }
        }
    }
    // metric weights of the stresses in the weak divergence
    const T W = PM ? pm->wij * pm->wk : a.w[i] * a.w[j] * a.w[k];
    gw[0] = W * rs * a.c1;
    gw[1] = W * rr * a.c2;
    gw[2] = W * (rr * rs) * a.c3;
    sn[0] = sxx; sn[1] = sxy; sn[2] = sxz; sn[3] = syy; sn[4] = syz; sn[5] = szz;
}

// point_stress, then the metric-weighted stresses for the weak divergence
// written to the flux slab `my` (9 x NP): entries 0, 3, 6 are contracted
// along x, 1, 4, 7 along y, 2, 5, 8 along z (point_divergence).
template <int N, typename T, int NSLS, bool ANISO, bool DU = false, bool SMEM = false, bool KS = false>
__device__ __forceinline__ void point_update(const StepArgs<T> &a, const T (&e)[9], T vx, T vy, T vz, int p, int i,
                                             int j, int k, int ex, int ey, int ez, T lam, T mu, T tau, T cA, T cB,
                                             T cC, const T (&sg)[6], const T (&m)[6][NSLS > 0 ? NSLS : 1], T *sig,
                                             T *mem, size_t cs, size_t nloc, T *my, T *du, T *sigc = nullptr) {
    constexpr int P = N + 1, NP = P * P * P;
    T sn[6], gw[3];
    point_stress<N, T, NSLS, ANISO, DU, SMEM, false, KS>(a, e, vx, vy, vz, i, j, k, ex, ey, ez, lam, mu, tau, cA, cB,
                                                         cC, sg, m, sig, mem, cs, nloc, du, sn, gw, nullptr, sigc);
    my[0 * NP + p] = sn[0] * gw[0];
    my[1 * NP + p] = sn[1] * gw[1];
    my[2 * NP + p] = sn[2] * gw[2];
    my[3 * NP + p] = sn[1] * gw[0];
    my[4 * NP + p] = sn[3] * gw[1];
    my[5 * NP + p] = sn[4] * gw[2];
    my[6 * NP + p] = sn[2] * gw[0];
    my[7 * NP + p] = sn[4] * gw[1];
    my[8 * NP + p] = sn[5] * gw[2];
}

// One element-local point of the step with CUDA-core contractions.
template <int N, typename T, int NSLS, bool ANISO, bool DU = false, bool KS = false>
__device__ __forceinline__ void point_step(const StepArgs<T> &a, const T *sD, const T *svx, const T *svy,
                                           const T *svz, int p, int i, int j, int k, int ex, int ey, int ez,
                                           T lam, T mu, T tau, T cA, T cB, T cC, const T (&sg)[6],
                                           const T (&m)[6][NSLS > 0 ? NSLS : 1], T *sig, T *mem, size_t cs,
                                           size_t nloc, T *my, T *du, T *sigc = nullptr) {
    T e[9];
    strain_contract<N, T>(sD, svx, svy, svz, i, j, k, e);
    point_update<N, T, NSLS, ANISO, DU, false, KS>(a, e, svx[p], svy[p], svz[p], p, i, j, k, ex, ey, ez, lam, mu, tau,
                                                   cA, cB, cC, sg, m, sig, mem, cs, nloc, my, du, sigc);
}

// Weak divergence at point (i,j,k): transposed line contractions over the
// element's flux slab `my` (9 x NP).
template <int N, typename T>
__device__ __forceinline__ void point_divergence(const T *Dt, const T *my, int i, int j, int k, T &fx, T &fy,
                                                 T &fz) {
    constexpr int P = N + 1, NP = P * P * P;
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const int px_ = q + P * (j + P * k);
        const int py_ = i + P * (q + P * k);
        const int pz_ = i + P * (j + P * q);
        const T di = Dt[i * P + q], dj = Dt[j * P + q], dk = Dt[k * P + q];
        fx += my[2 * NP + pz_] * dk + my[1 * NP + py_] * dj + my[0 * NP + px_] * di;
        fy += my[5 * NP + pz_] * dk + my[4 * NP + py_] * dj + my[3 * NP + px_] * di;
        fz += my[8 * NP + pz_] * dk + my[7 * NP + py_] * dj + my[6 * NP + px_] * di;
    }
}

template <int N>
__device__ __forceinline__ size_t unique_index(int NXU, int NYU, int ex, int ey, int ez, int i, int j, int k) {
    return (size_t)(ex * N + i) + (size_t)NXU * ((size_t)(ey * N + j) + (size_t)NYU * (size_t)(ez * N + k));
}

// One block per group of EPB elements and simulation.
template <int N, typename T, int NSLS, bool ANISO, bool DU, bool KS = false>
__global__ void __launch_bounds__(ElemCfg<N>::NT, sizeof(T) == 4 ? ElemCfg<N>::MINB : 1) k_element(const StepArgs<T> a) {
    constexpr int P = ElemCfg<N>::P, NP = ElemCfg<N>::NP, EPB = ElemCfg<N>::EPB, NT = ElemCfg<N>::NT;
    constexpr int MS = NSLS > 0 ? NSLS : 1;
    constexpr bool late_mem = SESNT_LATE_MEM < 0 ? N <= 5 : SESNT_LATE_MEM != 0;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sD = reinterpret_cast<T *>(smem_raw);  // [4][P*P]
    T *sv = sD + 4 * P * P;                   // [EPB][3][NP]
    T *sf = sv + EPB * 3 * NP;                // [EPB][9][NP]

    const int S = a.S;
    const int s = blockIdx.x % S;
    const int g = blockIdx.x / S;
    const int t = threadIdx.x;
    for (int x = t; x < 4 * P * P; x += NT) sD[x] = a.tabD[x];

    const int le = t / NP;
    const int p = t - le * NP;
    const int e = g * EPB + le;
    bool act = (le < EPB) && (e < a.nel);
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    int ex = 0, ey = 0, ez = 0;
    size_t u = 0;
    const size_t nuni = (size_t)a.nuni, nloc = (size_t)a.nloc;
    const size_t li = (size_t)e * NP + p;
    // Every global load of the step is issued before any store, so the loads
    // overlap each other and the line contractions: here, or for the memory
    // variables (late_mem) right after the barrier, which leaves the
    // scheduler fewer live registers while the velocities are staged.
    T lam = 0, mu = 0, tau = 0, cA = 0, cB = 0, cC = 0;
    T sg[6] = {0, 0, 0, 0, 0, 0};
    T m[6][MS];
    // stress and memory variables: element-blocked units (StateLayout)
    constexpr int NPS = StateLayout<NP, NSLS>::CS;
    constexpr size_t UNIT = StateLayout<NP, NSLS>::UNIT;
    const size_t sb = (size_t)e * S + s;
    T *sig = a.sig + sb * UNIT + p;
    T *mem = a.mem + sb * UNIT + p;
    act = act && in_range(unique_index<N>(a.NXU, a.NYU, e % a.nx, (e / a.nx) % a.ny, e / (a.nx * a.ny), i, j, k),
                          nuni, a.err) &&
          in_range(li, nloc, a.err) && in_range(sb * UNIT + 5 * NPS + p, (size_t)a.nel * S * UNIT, a.err) &&
          (NSLS == 0 || in_range(sb * UNIT + 6 * NPS + (6 * MS - 1) * NPS + p, (size_t)a.nel * S * UNIT, a.err));
    if (act) {
        ex = e % a.nx;
        ey = (e / a.nx) % a.ny;
        ez = e / (a.nx * a.ny);
        u = unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k);
        const T *vs = a.v + (size_t)s * 3 * nuni;
        const T vx = vs[u], vy = vs[nuni + u], vz = vs[2 * nuni + u];
        lam = ld_stream(a.lam + li);
        mu = ld_stream(a.mu + li);
        if constexpr (ANISO) {
            cA = ld_stream(a.A + li);
            cB = ld_stream(a.B + li);
            cC = ld_stream(a.C + li);
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) sg[c] = ld_stream(sig + c * NPS);
        if constexpr (NSLS > 0 && !late_mem) {
            tau = ld_stream(a.tau + li);
#pragma unroll
            for (int c = 0; c < 6; ++c)
#pragma unroll
                for (int q = 0; q < NSLS; ++q) m[c][q] = ld_stream(mem + (size_t)(c * NSLS + q) * NPS);
        }
        T *my = sv + le * 3 * NP;
        my[p] = vx;
        my[NP + p] = vy;
        my[2 * NP + p] = vz;
    }
    __syncthreads();
    if (act) {
        const T *svx = sv + le * 3 * NP;
        if constexpr (NSLS > 0 && late_mem) {
            tau = ld_stream(a.tau + li);
#pragma unroll
            for (int c = 0; c < 6; ++c)
#pragma unroll
                for (int q = 0; q < NSLS; ++q) m[c][q] = ld_stream(mem + (size_t)(c * NSLS + q) * NPS);
        }
        point_step<N, T, NSLS, ANISO, DU, KS>(a, sD, svx, svx + NP, svx + 2 * NP, p, i, j, k, ex, ey, ez, lam, mu,
                                              tau, cA, cB, cC, sg, m, sig, mem, NPS, nloc, sf + le * 9 * NP,
                                              DU ? a.du + (size_t)s * 9 * nloc + li : nullptr,
                                              KS ? a.sigc + sb * 6 * NPS + p : nullptr);
    }
    __syncthreads();
    if (act) {
        T fx = 0, fy = 0, fz = 0;
        point_divergence<N, T>(sD + 3 * P * P, sf + le * 9 * NP, i, j, k, fx, fy, fz);
        add_force(a, s, u, fx, fy, fz);
    }
}

// ---------------------------------------------------------------------------
// Batched elastic step with two simulations per thread (k_element_pair): the
// same element point of simulations s0 and s0+1 of the batch. The two share
// every derivative-table load of the line contractions, the metric, taper
// and quadrature factors, the material and the index arithmetic, which the
// batched elastic step is bound by (load/store and issue, not HBM). The
// per-simulation arithmetic and its order are those of k_element.
// ---------------------------------------------------------------------------
template <int N, typename T, bool ANISO>
__global__ void __launch_bounds__(ElemCfg<N>::NT, sizeof(T) == 4 ? ElemCfg<N>::MINB_PAIR : 1) k_element_pair(const StepArgs<T> a) {
    constexpr int P = ElemCfg<N>::P, NP = ElemCfg<N>::NP, EPB = ElemCfg<N>::EPB, NT = ElemCfg<N>::NT;
    constexpr int NPS = state_stride(NP);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sD = reinterpret_cast<T *>(smem_raw);  // [4][P*P]
    T *sv = sD + 4 * P * P;                   // [EPB][2][3][NP]
    T *sf = sv + EPB * 6 * NP;                // [EPB][2][9][NP]

    const int S = a.S, SP = S / 2;
    const int s0 = 2 * (blockIdx.x % SP);
    const int g = blockIdx.x / SP;
    const int t = threadIdx.x;
    for (int x = t; x < 4 * P * P; x += NT) sD[x] = a.tabD[x];

    const int le = t / NP;
    const int p = t - le * NP;
    const int e = g * EPB + le;
    bool act = (le < EPB) && (e < a.nel);
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    const size_t nuni = (size_t)a.nuni, nloc = (size_t)a.nloc;
    const size_t li = (size_t)e * NP + p;
    const size_t sb = (size_t)e * S + s0;  // simulation s0+1 follows at sb + 1
    T *sig0 = a.sig + sb * 6 * NPS + p;
    T *sig1 = sig0 + 6 * NPS;
    act = act && in_range(unique_index<N>(a.NXU, a.NYU, e % a.nx, (e / a.nx) % a.ny, e / (a.nx * a.ny), i, j, k),
                          nuni, a.err) &&
          in_range(li, nloc, a.err) && in_range((sb + 1) * 6 * NPS + 5 * NPS + p, (size_t)a.nel * S * 6 * NPS, a.err);
    int ex = 0, ey = 0, ez = 0;
    size_t u = 0;
    T lam = 0, mu = 0, cA = 0, cB = 0, cC = 0;
    T sg0[6] = {0, 0, 0, 0, 0, 0}, sg1[6] = {0, 0, 0, 0, 0, 0};
    T *v0 = sv + le * 6 * NP, *v1 = v0 + 3 * NP;
    if (act) {  // every global load first, as in k_element
        ex = e % a.nx;
        ey = (e / a.nx) % a.ny;
        ez = e / (a.nx * a.ny);
        u = unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k);
        const T *va = a.v + (size_t)s0 * 3 * nuni, *vb = va + 3 * nuni;
        const T ax = va[u], ay = va[nuni + u], az = va[2 * nuni + u];
        const T bx = vb[u], by = vb[nuni + u], bz = vb[2 * nuni + u];
        lam = ld_stream(a.lam + li);
        mu = ld_stream(a.mu + li);
        if constexpr (ANISO) {
            cA = ld_stream(a.A + li);
            cB = ld_stream(a.B + li);
            cC = ld_stream(a.C + li);
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            sg0[c] = ld_stream(sig0 + c * NPS);
            sg1[c] = ld_stream(sig1 + c * NPS);
        }
        v0[p] = ax;
        v0[NP + p] = ay;
        v0[2 * NP + p] = az;
        v1[p] = bx;
        v1[NP + p] = by;
        v1[2 * NP + p] = bz;
    }
    __syncthreads();
    if (act) {
        // line contractions of both simulations with one set of table loads
        T e0[9], e1[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) e0[c] = e1[c] = 0;
        const T *Dx = sD, *Dy = sD + P * P, *Dz = sD + 2 * P * P;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int px_ = q + P * (j + P * k), py_ = i + P * (q + P * k), pz_ = i + P * (j + P * q);
            const T dx = Dx[q * P + i], dy = Dy[q * P + j], dz = Dz[q * P + k];
            e0[0] += v0[px_] * dx;
            e0[1] += v0[NP + px_] * dx;
            e0[2] += v0[2 * NP + px_] * dx;
            e0[3] += v0[py_] * dy;
            e0[4] += v0[NP + py_] * dy;
            e0[5] += v0[2 * NP + py_] * dy;
            e0[6] += v0[pz_] * dz;
            e0[7] += v0[NP + pz_] * dz;
            e0[8] += v0[2 * NP + pz_] * dz;
            e1[0] += v1[px_] * dx;
            e1[1] += v1[NP + px_] * dx;
            e1[2] += v1[2 * NP + px_] * dx;
            e1[3] += v1[py_] * dy;
            e1[4] += v1[NP + py_] * dy;
            e1[5] += v1[2 * NP + py_] * dy;
            e1[6] += v1[pz_] * dz;
            e1[7] += v1[NP + pz_] * dz;
            e1[8] += v1[2 * NP + pz_] * dz;
        }
        T g0[9], g1[9];
        complete_gradient<N, T>(a, e0, v0[p], v0[NP + p], v0[2 * NP + p], i, k, ex, ez, g0);
        complete_gradient<N, T>(a, e1, v1[p], v1[NP + p], v1[2 * NP + p], i, k, ex, ez, g1);
        const T tp = taper_value(a.px[ex * P + i], a.py[ey * P + j], a.pz[ez * P + k], a.inv_alpha);
        const T rr = a.r[ez * P + k];
        const T rs = rr * a.sin_t[ex * P + i];
        const T W = a.w[i] * a.w[j] * a.w[k];
        const T gx = W * rs * a.c1, gy = W * rr * a.c2, gz = W * (rr * rs) * a.c3;
        const T m[6][1] = {{0}, {0}, {0}, {0}, {0}, {0}};
        auto update = [&](const T(&gg)[9], const T(&sg)[6], T *sig, T *my) {
            const T exx = gg[kDuXX], eyy = gg[kDuYY], ezz = gg[kDuZZ];
            const T exy = (gg[kDuXY] + gg[kDuYX]) * T(0.5);
            const T exz = (gg[kDuXZ] + gg[kDuZX]) * T(0.5);
            const T eyz = (gg[kDuYZ] + gg[kDuZY]) * T(0.5);
            T rxx, ryy, rzz, rxy, rxz, ryz;
            stress_rates<T, 0, ANISO>(exx, eyy, ezz, exy, exz, eyz, lam, mu, T(0), cA, cB, cC, m, rxx, ryy, rzz, rxy,
                                      rxz, ryz);
            const T sxx = sg[0] + a.dt * rxx;
            const T sxy = sg[1] + a.dt * rxy;
            const T sxz = sg[2] + a.dt * rxz;
            const T syy = sg[3] + a.dt * ryy;
            const T syz = sg[4] + a.dt * ryz;
            const T szz = sg[5] + a.dt * rzz;
            st_stream(sig, sxx * tp);
            st_stream(sig + NPS, sxy * tp);
            st_stream(sig + 2 * NPS, sxz * tp);
            st_stream(sig + 3 * NPS, syy * tp);
            st_stream(sig + 4 * NPS, syz * tp);
            st_stream(sig + 5 * NPS, szz * tp);
            my[0 * NP + p] = sxx * gx;
            my[1 * NP + p] = sxy * gy;
            my[2 * NP + p] = sxz * gz;
            my[3 * NP + p] = sxy * gx;
            my[4 * NP + p] = syy * gy;
            my[5 * NP + p] = syz * gz;
            my[6 * NP + p] = sxz * gx;
            my[7 * NP + p] = syz * gy;
            my[8 * NP + p] = szz * gz;
        };
        update(g0, sg0, sig0, sf + le * 18 * NP);
        update(g1, sg1, sig1, sf + le * 18 * NP + 9 * NP);
    }
    __syncthreads();
    if (act) {
        const T *f0 = sf + le * 18 * NP, *f1 = f0 + 9 * NP, *Dt = sD + 3 * P * P;
        T ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int px_ = q + P * (j + P * k), py_ = i + P * (q + P * k), pz_ = i + P * (j + P * q);
            const T di = Dt[i * P + q], dj = Dt[j * P + q], dk = Dt[k * P + q];
            ax += f0[2 * NP + pz_] * dk + f0[1 * NP + py_] * dj + f0[0 * NP + px_] * di;
            ay += f0[5 * NP + pz_] * dk + f0[4 * NP + py_] * dj + f0[3 * NP + px_] * di;
            az += f0[8 * NP + pz_] * dk + f0[7 * NP + py_] * dj + f0[6 * NP + px_] * di;
            bx += f1[2 * NP + pz_] * dk + f1[1 * NP + py_] * dj + f1[0 * NP + px_] * di;
            by += f1[5 * NP + pz_] * dk + f1[4 * NP + py_] * dj + f1[3 * NP + px_] * di;
            bz += f1[8 * NP + pz_] * dk + f1[7 * NP + py_] * dj + f1[6 * NP + px_] * di;
        }
        add_force(a, s0, u, ax, ay, az);
        add_force(a, s0 + 1, u, bx, by, bz);
    }
}


// Source slabs through the weak divergence, one block per resolved
// (simulation, element) record. The slab set after step it-1 acts in step it
// (src/ses3d-nt.F90:240-250), so step 1 injects nothing.
template <int N, typename T>
__global__ void __launch_bounds__(((ElemCfg<N>::NP + 31) / 32) * 32) k_sources(const StepArgs<T> a) {
    constexpr int P = ElemCfg<N>::P, NP = ElemCfg<N>::NP;
    const int it = *a.d_it + a.step_off;
    if (it < 2) return;
    const int di = it - 2;  // data(it-1), 0-based
    __shared__ T sf[9 * NP];
    __shared__ T sD[P * P];
    const SrcRec rec = a.src[blockIdx.x];
    const int t = threadIdx.x;
    for (int x = t; x < P * P; x += blockDim.x) sD[x] = a.tabD[3 * P * P + x];
    const int p = t;
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    const int e = rec.elem;
    const int ex = e % a.nx, ey = (e / a.nx) % a.ny, ez = e / (a.nx * a.ny);
    bool act = p < NP && in_range(e, a.nel, a.err) && in_range(rec.sim, a.S, a.err) && in_range(di, a.nt, a.err);
    for (int c = 0; c < 9 && act; ++c)
        act = rec.vm[c] < 0 || (in_range(rec.vm[c], a.n_src_vm, a.err) && in_range(rec.data[c], a.n_src_data, a.err));
    T f0[3] = {0, 0, 0};
    if (act) {
        const T rr = a.r[ez * P + k];
        const T rs = rr * a.sin_t[ex * P + i];
        const T W = a.w[i] * a.w[j] * a.w[k];
        const T rr2 = rr * rs;
        T m[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            m[c] = 0;
            if (rec.vm[c] >= 0) {
                const T d = a.src_data[(size_t)rec.data[c] * a.nt + di];
                m[c] = (-d * a.src_vm[(size_t)rec.vm[c] * NP + p]) / (a.jac * W * rr2);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (rec.vm[6 + c] >= 0) {
                const T d = a.src_data[(size_t)rec.data[6 + c] * a.nt + di];
                f0[c] = -d * a.src_vm[(size_t)rec.vm[6 + c] * NP + p];
            }
        const T gx = W * rs * a.c1, gy = W * rr * a.c2, gz = W * rr2 * a.c3;
        // m = xx, xy, xz, yy, yz, zz
        sf[0 * NP + p] = m[0] * gx;
        sf[1 * NP + p] = m[1] * gy;
        sf[2 * NP + p] = m[2] * gz;
        sf[3 * NP + p] = m[1] * gx;
        sf[4 * NP + p] = m[3] * gy;
        sf[5 * NP + p] = m[4] * gz;
        sf[6 * NP + p] = m[2] * gx;
        sf[7 * NP + p] = m[4] * gy;
        sf[8 * NP + p] = m[5] * gz;
    }
    __syncthreads();
    if (!act) return;
    T fx = f0[0], fy = f0[1], fz = f0[2];
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const int px_ = q + P * (j + P * k);
        const int py_ = i + P * (q + P * k);
        const int pz_ = i + P * (j + P * q);
        const T dI = sD[i * P + q], dJ = sD[j * P + q], dK = sD[k * P + q];
        fx += sf[2 * NP + pz_] * dK + sf[1 * NP + py_] * dJ + sf[0 * NP + px_] * dI;
        fy += sf[5 * NP + pz_] * dK + sf[4 * NP + py_] * dJ + sf[3 * NP + px_] * dI;
        fz += sf[8 * NP + pz_] * dK + sf[7 * NP + py_] * dJ + sf[6 * NP + px_] * dI;
    }
    const size_t nuni = (size_t)a.nuni;
    const size_t u =
        (size_t)(ex * N + i) + (size_t)a.NXU * ((size_t)(ey * N + j) + (size_t)a.NYU * (size_t)(ez * N + k));
    add_force(a, rec.sim, u, fx, fy, fz);
}

// Decode a unique point into the element-local copy with the lowest element
// index along each axis (the copy whose 1-D tables the node kernel reads).
template <int N>
__device__ __forceinline__ void unique_to_local(unsigned g, int ne, int &e, int &n) {
    e = min((int)(g / N), ne - 1);
    n = (int)g - e * N;
}

template <int N, typename T, bool KAHAN>
__global__ void __launch_bounds__(256) k_node(const StepArgs<T> a) {
    constexpr int P = N + 1;
    const unsigned u = blockIdx.x * 256u + threadIdx.x;
    const int s = blockIdx.y;
    if (u >= (unsigned)a.nuni) return;
    const size_t nuni = (size_t)a.nuni;
    T *__restrict__ F = a.F + (size_t)s * 3 * nuni + u;
    T *__restrict__ v = a.v + (size_t)s * 3 * nuni + u;
    T *__restrict__ vc = KAHAN ? a.vc + (size_t)s * 3 * nuni + u : nullptr;
    double *__restrict__ F64 = a.F64 ? a.F64 + (size_t)s * 3 * nuni + u : nullptr;
    // all loads before any store (stores to possibly aliasing arrays would
    // otherwise serialise each thread's later loads behind them)
    T f[3], vo[3], co[3] = {0, 0, 0};
    double fd[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (F64) fd[c] = F64[c * nuni];
        else f[c] = F[c * nuni];
        vo[c] = v[c * nuni];
        if constexpr (KAHAN) co[c] = vc[c * nuni];
    }
    const T im = a.invM[u];
    const unsigned gx = u % (unsigned)a.NXU, rest = u / (unsigned)a.NXU;
    const unsigned gy = rest % (unsigned)a.NYU, gz = rest / (unsigned)a.NYU;
    int ex, i, ey, j, ez, k;
    unique_to_local<N>(gx, a.nx, ex, i);
    unique_to_local<N>(gy, a.ny, ey, j);
    unique_to_local<N>(gz, a.nz, ez, k);
    const T tp = taper_value(a.px[ex * P + i], a.py[ey * P + j], a.pz[ez * P + k], a.inv_alpha);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        T acc;
        if (F64) {
            F64[c * nuni] = 0.0;
            acc = (T)(fd[c] * (double)im);  // the FP64 force rounded once, with the mass divide
        } else {
            F[c * nuni] = T(0);
            acc = f[c] * im;
        }
        if constexpr (KAHAN) {
            // Kahan-compensated v += dt*acc (the compensation is tapered with v)
            const T y = a.dt * acc - co[c];
            const T tsum = vo[c] + y;
            vc[c * nuni] = ((tsum - vo[c]) - y) * tp;
            v[c * nuni] = tsum * tp;
        } else {
            v[c * nuni] = (vo[c] + a.dt * acc) * tp;
        }
    }
}

}  // namespace sesnt

#include "channels.cuh"

namespace sesnt {

template <int N, typename T>
__global__ void __launch_bounds__(128) k_receivers(const StepArgs<T> a) {
    constexpr int P = N + 1, NP = P * P * P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * 4 + warp;
    const int s = blockIdx.y;
    if (r >= a.nrec) return;
    const int it = *a.d_it + a.step_off;
    const int e = a.rec_elem[r];
    if (!in_range(e, a.nel, a.err) || !in_range(it - 1, a.nt, a.err)) return;  // whole warp
    const int ex = e % a.nx, ey = (e / a.nx) % a.ny, ez = e / (a.nx * a.ny);
    const size_t nuni = (size_t)a.nuni;
    const T *vs = a.v + (size_t)s * 3 * nuni;
    const T *vm = a.rec_vm + (size_t)r * NP;
    T acc[3] = {0, 0, 0};
    for (int p = lane; p < NP; p += 32) {
        const int i = p % P, j = (p / P) % P, k = p / (P * P);
        const size_t u =
            (size_t)(ex * N + i) + (size_t)a.NXU * ((size_t)(ey * N + j) + (size_t)a.NYU * (size_t)(ez * N + k));
        const T wgt = vm[p];
        acc[0] += wgt * vs[u];
        acc[1] += wgt * vs[nuni + u];
        acc[2] += wgt * vs[2 * nuni + u];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        T x = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        acc[c] = x;
    }
    if (lane == 0) {
        const size_t at = (((size_t)s * a.nrec + r) * 3) * a.nt + (it - 1);
        T *out = a.seis + at;
        out[0] = acc[0];
        out[(size_t)a.nt] = acc[1];
        out[2 * (size_t)a.nt] = acc[2];
        if (a.seis_host) {
            // host-mapped copy read by sesnt_get_samples without a device copy
            float *h = a.seis_host + at;
            h[0] = (float)acc[0];
            h[(size_t)a.nt] = (float)acc[1];
            h[2 * (size_t)a.nt] = (float)acc[2];
        }
    }
    if (a.rec_xmask) record_extra<N, T>(a, r, s, it, lane, ex, ey, ez, vm);
}

// Inverse assembled mass matrix in FP64 (src/model_paras.F90:410-415):
// MM = -jac * r^2 * sin(theta) * rho * w_i w_j w_k summed over the copies of
// each unique point, rho = 1/rhoinv where rhoinv > 0 else 0.
// sin_t and r come in double from the caller's tables (dsin, dr).
template <int N, typename T>
__global__ void __launch_bounds__(256) k_inv_mass(const StepArgs<T> a, const T *rhoinv, const double *dsin,
                                                  const double *dr, const double *dw, double jac) {
    constexpr int P = N + 1, NP = P * P * P;
    const unsigned u = blockIdx.x * 256u + threadIdx.x;
    if (u >= (unsigned)a.nuni) return;
    const int g[3] = {(int)(u % (unsigned)a.NXU), (int)((u / (unsigned)a.NXU) % (unsigned)a.NYU),
                      (int)(u / ((unsigned)a.NXU * (unsigned)a.NYU))};
    const int ne[3] = {a.nx, a.ny, a.nz};
    int ce[3][2], cn[3][2], cnt[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int e0 = g[d] / N, n0 = g[d] - e0 * N;
        if (n0 == 0 && e0 > 0 && e0 < ne[d]) {
            cnt[d] = 2;
            ce[d][0] = e0 - 1; cn[d][0] = N;
            ce[d][1] = e0;     cn[d][1] = 0;
        } else {
            cnt[d] = 1;
            ce[d][0] = min(e0, ne[d] - 1);
            cn[d][0] = g[d] - ce[d][0] * N;
        }
    }
    double mm = 0.0;
    for (int c2 = 0; c2 < cnt[2]; ++c2)
        for (int c1 = 0; c1 < cnt[1]; ++c1)
            for (int c0 = 0; c0 < cnt[0]; ++c0) {
                const int ex = ce[0][c0], i = cn[0][c0], ey = ce[1][c1], j = cn[1][c1], ez = ce[2][c2], k = cn[2][c2];
                const size_t e = (size_t)ex + (size_t)a.nx * (ey + (size_t)a.ny * ez);
                const double ri = (double)rhoinv[e * NP + i + P * (j + P * k)];
                const double rho = ri > 0.0 ? 1.0 / ri : 0.0;
                const double rr = dr[ez * P + k];
                mm += -(jac * rr * rr * dsin[ex * P + i] * rho * (dw[i] * dw[j] * dw[k]));
            }
    const_cast<T *>(a.invM)[u] = (T)(1.0 / mm);
}

template <int N, typename T>
__global__ void __launch_bounds__(256) k_gather_local(const StepArgs<T> a, const T *uni, T *loc) {
    constexpr int P = N + 1, NP = P * P * P;
    const size_t li = (size_t)blockIdx.x * 256 + threadIdx.x;
    if (li >= (size_t)a.nloc) return;
    const size_t e = li / NP;
    const int p = (int)(li - e * NP);
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    const int ex = (int)(e % a.nx), ey = (int)((e / a.nx) % a.ny), ez = (int)(e / ((size_t)a.nx * a.ny));
    const size_t u =
        (size_t)(ex * N + i) + (size_t)a.NXU * ((size_t)(ey * N + j) + (size_t)a.NYU * (size_t)(ez * N + k));
    loc[li] = uni[u];
}

template <int N, typename T>
__global__ void __launch_bounds__(256) k_scatter_unique(const StepArgs<T> a, const T *loc, T *uni) {
    constexpr int P = N + 1, NP = P * P * P;
    const size_t li = (size_t)blockIdx.x * 256 + threadIdx.x;
    if (li >= (size_t)a.nloc) return;
    const size_t e = li / NP;
    const int p = (int)(li - e * NP);
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    const int ex = (int)(e % a.nx), ey = (int)((e / a.nx) % a.ny), ez = (int)(e / ((size_t)a.nx * a.ny));
    const size_t u =
        (size_t)(ex * N + i) + (size_t)a.NXU * ((size_t)(ey * N + j) + (size_t)a.NYU * (size_t)(ez * N + k));
    atomicAdd(uni + u, loc[li]);
}

template <int N, typename T>
__global__ void __launch_bounds__(256) k_taper_local(const StepArgs<T> a, T *loc) {
    constexpr int P = N + 1, NP = P * P * P;
    const size_t li = (size_t)blockIdx.x * 256 + threadIdx.x;
    if (li >= (size_t)a.nloc) return;
    const size_t e = li / NP;
    const int p = (int)(li - e * NP);
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    const int ex = (int)(e % a.nx), ey = (int)((e / a.nx) % a.ny), ez = (int)(e / ((size_t)a.nx * a.ny));
    loc[li] = taper_value(a.px[ex * P + i], a.py[ey * P + j], a.pz[ez * P + k], a.inv_alpha);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
constexpr size_t kMaxSmemPerBlock = 227 * 1024;

template <int N, typename T, int NSLS, bool ANISO>
int launch_element_v(const StepArgs<T> &a, void *stream) {
    using C = ElemCfg<N>;
    const long long groups = (long long)((a.nel + C::EPB - 1) / C::EPB) * a.S;
    if constexpr (NSLS == 0) {
        if (a.S >= 2 && a.S % 2 == 0 && !a.du && a.pair) {
            const size_t smem2 = sizeof(T) * (4 * C::P * C::P + C::EPB * 24 * C::NP);
            k_element_pair<N, T, ANISO><<<(unsigned)(groups / 2), C::NT, smem2, (cudaStream_t)stream>>>(a);
            return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
        }
    }
    const size_t smem = sizeof(T) * (4 * C::P * C::P + C::EPB * 12 * C::NP);
    if (a.du) k_element<N, T, NSLS, ANISO, true><<<(unsigned)groups, C::NT, smem, (cudaStream_t)stream>>>(a);
    else if (a.sigc) k_element<N, T, NSLS, ANISO, false, true><<<(unsigned)groups, C::NT, smem, (cudaStream_t)stream>>>(a);
    else k_element<N, T, NSLS, ANISO, false><<<(unsigned)groups, C::NT, smem, (cudaStream_t)stream>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int N, typename T, int NSLS, bool ANISO>
int prepare_variant() {
    using C = ElemCfg<N>;
    const size_t smem = sizeof(T) * (4 * C::P * C::P + C::EPB * 12 * C::NP);
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024)
        e = cudaFuncSetAttribute(k_element<N, T, NSLS, ANISO, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
    if (e == cudaSuccess && smem > 48 * 1024)
        e = cudaFuncSetAttribute(k_element<N, T, NSLS, ANISO, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
    if (e == cudaSuccess && smem > 48 * 1024)
        e = cudaFuncSetAttribute(k_element<N, T, NSLS, ANISO, false, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if constexpr (NSLS == 0) {
        const size_t smem2 = sizeof(T) * (4 * C::P * C::P + C::EPB * 24 * C::NP);
        if (e == cudaSuccess && smem2 > 48 * 1024)
            e = cudaFuncSetAttribute(k_element_pair<N, T, ANISO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem2);
    }
    return e == cudaSuccess ? 0 : -1;
}

}  // namespace sesnt

#include "element_tc.cuh"
#include "element_tma.cuh"
#include "element_cols.cuh"

namespace sesnt {

// Kernel attributes (large dynamic shared memory) and the resident-block
// counts of the persistent kernel, once per handle, outside stream capture.
template <int N, typename T>
int prepare_element() {
    if (prepare_variant<N, T, 0, false>() || prepare_variant<N, T, 0, true>() ||
        prepare_variant<N, T, kNsls, false>() || prepare_variant<N, T, kNsls, true>())
        return -1;
    if constexpr (std::is_same_v<T, float>)
        if (prepare_element_tc<N, 1>() || prepare_element_tc<N, 2>()) return -1;
    if (prepare_element_tma<N, T, 0, false>() || prepare_element_tma<N, T, 0, true>() ||
        prepare_element_tma<N, T, kNsls, false>() || prepare_element_tma<N, T, kNsls, true>())
        return -1;
    if constexpr (ElemCfg<N>::EPB == 1)
        if (prepare_element_stage<N, T, kNsls, false>() || prepare_element_stage<N, T, kNsls, true>()) return -1;
    if (prepare_element_cols<N, T, false>() || prepare_element_cols<N, T, true>()) return -1;
    return 0;
}


// TMA-fed persistent kernel (SESNT_FLAG_PERSISTENT_ELEMENT); 1 when this
// configuration has none.
template <int N, typename T>
int launch_element_bulk(const StepArgs<T> &a, bool sls, bool aniso, void *stream) {
    if (sls) return aniso ? launch_element_tma<N, T, kNsls, true>(a, stream) : launch_element_tma<N, T, kNsls, false>(a, stream);
    return aniso ? launch_element_tma<N, T, 0, true>(a, stream) : launch_element_tma<N, T, 0, false>(a, stream);
}

// The element kernel one step launches, decided on the host from the
// handle's configuration (plan_element) so that the launcher, the tuner and
// the kernel name a caller reads agree.
enum class ElemKernel : int { Tc, Point, Pair, StageBulk, StageReg, Persistent, Columns, ColumnsStaged, ColumnsPair };

inline const char *elem_kernel_name(ElemKernel k) {
    switch (k) {
        case ElemKernel::Tc: return "k_element_tc";
        case ElemKernel::Point: return "k_element";
        case ElemKernel::Pair: return "k_element_pair";
        case ElemKernel::StageBulk: return "k_element_stage";
        case ElemKernel::StageReg: return "k_element_stage (register stores)";
        case ElemKernel::Persistent: return "k_element_tma";
        case ElemKernel::Columns: return "k_element_cols";
        case ElemKernel::ColumnsStaged: return "k_element_cols (staged stress)";
        case ElemKernel::ColumnsPair: return "k_element_cols2";
    }
    return "?";
}

template <int N, typename T>
bool has_persistent(bool sls, bool aniso) {
    using C0 = TmaCfg<N, T, 0>;
    using C3 = TmaCfg<N, T, kNsls>;
    if (sls) {
        if (C3::SMEM > kMaxSmemPerBlock) return false;
        return (aniso ? TmaLaunch<N, T, kNsls, true>::blocks : TmaLaunch<N, T, kNsls, false>::blocks) > 0;
    }
    if (C0::SMEM > kMaxSmemPerBlock) return false;
    return (aniso ? TmaLaunch<N, T, 0, true>::blocks : TmaLaunch<N, T, 0, false>::blocks) > 0;
}

template <int N, typename T>
constexpr bool has_staged() {
    return ElemCfg<N>::EPB == 1 && StageCfg<N, T, kNsls>::SMEM <= kMaxSmemPerBlock;
}

template <int N, typename T>
constexpr bool has_columns(bool stage) {
    return ColCfg<N>::template smem<T>(stage) <= kMaxSmemPerBlock;
}

template <int N, typename T>
constexpr bool has_columns2() {
    return ColCfg<N>::template smem2<T>() <= kMaxSmemPerBlock;
}

// A variant chosen by the tuner or the caller (StepArgs::variant) where the
// configuration has it; otherwise the rules: tensor-core contractions when
// asked for; the persistent kernel when asked for; the staged kernel for SLS
// steps of degrees 4-7 (at degree 4 in FP32 with the L2 prefetch half a
// resident wave ahead, StepArgs::prefetch); one point per thread, with paired
// simulations for even elastic batches. The displacement gradient (du) is kept only by
// k_element.
template <int N, typename T>
ElemKernel plan_element(const StepArgs<T> &a, bool sls, bool aniso) {
    if (std::is_same_v<T, float> && a.contraction) return ElemKernel::Tc;
    const bool even = a.S >= 2 && a.S % 2 == 0;
    if (a.du) return ElemKernel::Point;
    // compensated stress integration: the staged kernel with register stores
    // (SLS, degrees 4-7) or one point per thread
    if (a.sigc) return sls && has_staged<N, T>() ? ElemKernel::StageReg : ElemKernel::Point;
    switch (a.variant) {
        case kVarPoint: return ElemKernel::Point;
        case kVarPair: if (!sls && even) return ElemKernel::Pair; break;
        case kVarStage: if (sls && has_staged<N, T>()) return ElemKernel::StageBulk; break;
        case kVarStageReg: if (sls && has_staged<N, T>()) return ElemKernel::StageReg; break;
        case kVarPersistent: if (has_persistent<N, T>(sls, aniso)) return ElemKernel::Persistent; break;
        case kVarColumns: if (!sls && has_columns<N, T>(false)) return ElemKernel::Columns; break;
        case kVarColumnsStaged: if (!sls && has_columns<N, T>(true)) return ElemKernel::ColumnsStaged; break;
        case kVarColumnsPair: if (!sls && even && has_columns2<N, T>()) return ElemKernel::ColumnsPair; break;
        default: break;
    }
    if (a.persistent && has_persistent<N, T>(sls, aniso)) return ElemKernel::Persistent;
    if (sls && a.stage && has_staged<N, T>())
        return StageCfg<N, T, kNsls>::STORE_DEFAULT ? ElemKernel::StageBulk : ElemKernel::StageReg;
    if (!sls && even && a.pair) return ElemKernel::Pair;
    return ElemKernel::Point;
}

template <int N, typename T>
const char *element_name(const StepArgs<T> &a, bool sls, bool aniso) {
    return elem_kernel_name(plan_element<N, T>(a, sls, aniso));
}

template <int N, typename T>
int launch_element(const StepArgs<T> &a, bool sls, bool aniso, void *stream) {
    const ElemKernel k = plan_element<N, T>(a, sls, aniso);
    StepArgs<T> b = a;
    switch (k) {
        case ElemKernel::Tc:
            if constexpr (std::is_same_v<T, float>) return launch_element_tc<N>(a, sls, aniso, stream);
            return -1;
        case ElemKernel::Persistent: {
            const int r = launch_element_bulk<N, T>(a, sls, aniso, stream);
            return r > 0 ? -1 : r;
        }
        case ElemKernel::StageBulk:
        case ElemKernel::StageReg:
            if constexpr (ElemCfg<N>::EPB == 1) {
                const int store = k == ElemKernel::StageBulk ? 1 : 0;
                // the wait mode (variant_arg) only where the staged kernel was chosen
                if (a.variant != kVarStage && a.variant != kVarStageReg) b.variant_arg = 0;
                const int r = aniso ? launch_element_stage<N, T, kNsls, true>(b, store, stream)
                                    : launch_element_stage<N, T, kNsls, false>(b, store, stream);
                return r > 0 ? -1 : r;
            }
            return -1;
        case ElemKernel::Columns: {
            const int r = aniso ? launch_element_cols<N, T, true, false>(a, a.variant_arg & 3, stream)
                                : launch_element_cols<N, T, false, false>(a, a.variant_arg & 3, stream);
            return r > 0 ? -1 : r;
        }
        case ElemKernel::ColumnsStaged: {
            const int r = aniso ? launch_element_cols<N, T, true, true>(a, a.variant_arg & 3, stream)
                                : launch_element_cols<N, T, false, true>(a, a.variant_arg & 3, stream);
            return r > 0 ? -1 : r;
        }
        case ElemKernel::ColumnsPair: {
            const int r = aniso ? launch_element_cols2<N, T, true>(a, a.variant_arg & 3, stream)
                                : launch_element_cols2<N, T, false>(a, a.variant_arg & 3, stream);
            return r > 0 ? -1 : r;
        }
        case ElemKernel::Pair: b.pair = 1; break;
        case ElemKernel::Point: b.pair = 0; break;
    }
    if (sls) return aniso ? launch_element_v<N, T, kNsls, true>(b, stream) : launch_element_v<N, T, kNsls, false>(b, stream);
    return aniso ? launch_element_v<N, T, 0, true>(b, stream) : launch_element_v<N, T, 0, false>(b, stream);
}

template <int N, typename T>
int launch_node(const StepArgs<T> &a, bool kahan, void *stream) {
    dim3 grid((unsigned)((a.nuni + 255) / 256), (unsigned)a.S);
    if (kahan) k_node<N, T, true><<<grid, 256, 0, (cudaStream_t)stream>>>(a);
    else k_node<N, T, false><<<grid, 256, 0, (cudaStream_t)stream>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int N, typename T>
int launch_sources(const StepArgs<T> &a, void *stream) {
    if (a.nsrc <= 0) return 0;
    constexpr int NT = ((ElemCfg<N>::NP + 31) / 32) * 32;
    k_sources<N, T><<<a.nsrc, NT, 0, (cudaStream_t)stream>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int N, typename T>
int launch_receivers(const StepArgs<T> &a, void *stream) {
    if (a.nrec <= 0) return 0;
    dim3 grid((unsigned)((a.nrec + 3) / 4), (unsigned)a.S);
    k_receivers<N, T><<<grid, 128, 0, (cudaStream_t)stream>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int N, typename T>
int launch_gather_local(const StepArgs<T> &a, const T *uni, T *loc, void *stream) {
    k_gather_local<N, T><<<(unsigned)((a.nloc + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a, uni, loc);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int N, typename T>
int launch_scatter_unique(const StepArgs<T> &a, const T *loc, T *uni, void *stream) {
    k_scatter_unique<N, T><<<(unsigned)((a.nloc + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a, loc, uni);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int N, typename T>
int launch_taper_local(const StepArgs<T> &a, T *loc, void *stream) {
    k_taper_local<N, T><<<(unsigned)((a.nloc + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a, loc);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sesnt

namespace sesnt {

template <int N, typename T>
int launch_inv_mass(const StepArgs<T> &a, const T *rhoinv, const double *dsin, const double *dr, const double *dw,
                    double jac, void *stream) {
    k_inv_mass<N, T><<<(unsigned)((a.nuni + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a, rhoinv, dsin, dr, dw,
                                                                                         jac);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int N, typename T>
const LpdOps<T> *lpd_ops_n() {
    static const LpdOps<T> ops = {
        &launch_element<N, T>,        &launch_node<N, T>,        &launch_sources<N, T>,
        &launch_receivers<N, T>,      &launch_inv_mass<N, T>,    &launch_gather_local<N, T>,
        &launch_scatter_unique<N, T>, &launch_taper_local<N, T>, &launch_rot_strain<N, T>,
        &launch_derived<N, T>,        &prepare_element<N, T>,    &element_name<N, T>,       ElemCfg<N>::NT,
        sizeof(T) * (4 * ElemCfg<N>::P * ElemCfg<N>::P + ElemCfg<N>::EPB * 12 * ElemCfg<N>::NP)};
    return &ops;
}

}  // namespace sesnt

// One translation unit per degree instantiates everything for FP32 and FP64.
#define SESNT_INSTANTIATE_LPD(NN)                                    \
    namespace sesnt {                                                \
    template const LpdOps<float> *lpd_ops_n<NN, float>();            \
    template const LpdOps<double> *lpd_ops_n<NN, double>();          \
    }
