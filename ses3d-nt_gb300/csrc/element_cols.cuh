// Elastic element kernel with one thread per (i, j) column of an element
// (k_element_cols), for batched elastic steps. A block holds G (element,
// simulation) units, consecutive in the element-major state order, and each
// unit's P*P threads own its columns: a thread keeps its column's velocity
// (3 x P values) and its z-direction fluxes (3 x P) in registers, so the
// z line contractions of the strain (src/evolution.f90:136-144) and of the
// weak divergence (:350-356) read no shared memory: their derivative-table
// entries have compile-time indices and are read from the launch parameters
// (StepArgs::tabz) as constant-bank operands. Only the x and y
// contractions go through per-unit slabs: per point and simulation that is
// 3 velocity stores + 30 loads and 6 flux stores + 30 loads, against 12
// stores + 90 loads with one thread per point (k_element, k_element_pair),
// whose batched elastic launches were bound by the shared-memory data pipe
// (L1 90% busy, 36 M wavefronts on the 12x12x8 grid with 64 simulations).
// The derivative-table columns a thread contracts with (x and y, strain and
// divergence) sit in registers. Per point, the arithmetic and its
// order are those of k_element (strain_contract, point_stress,
// point_divergence).
#pragma once

namespace sesnt {

template <int N>
struct ColCfg {
    static constexpr int P = N + 1, PP = P * P, NP = P * P * P;
    static_assert(PP <= 64, "the z tables of the launch parameters hold 64 values");
    // units per block: as many whole columns sets as fit 128 threads
    static constexpr int G = PP <= 128 ? 128 / PP : 1;
    static constexpr int NT = ((G * PP + 31) / 32) * 32;
    // Shared-memory stride of one unit's slabs (v, x fluxes, y fluxes:
    // 9 x NP values), padded so that it is congruent to PP modulo the 32
    // banks: thread t = unit*PP + c then finds the element c of its unit's
    // slab in bank t mod 32 (for 4-byte values), and the two units a warp
    // spans never meet in a bank on the stores, the y-line loads or the
    // x-line loads. Unpadded (9*125 = 1125 = 5 mod 32 at degree 4) a third
    // of the shared-memory wavefronts were bank conflicts.
    static constexpr int US = 9 * NP + ((PP - 9 * NP) % 32 + 32) % 32;
    static constexpr size_t SMEM_T = 4 * PP + (size_t)G * US;  // values of T: tables, slabs
    static constexpr int NPS = state_stride(NP);
    // STAGE: the stress of the block's G units (one contiguous range of the
    // element-major state, 6 x NPS values per unit) follows, 128-byte
    // aligned, one unit every SS values, then the mbarrier. SS is padded to
    // a multiple of 16 bytes near PP modulo 32 banks (the same reason as US;
    // 6 x 128 = 0 mod 32 at degree 4 put every unit's column c in one bank).
    template <typename T>
    SESNT_HD static constexpr int stage_stride() {
        constexpr int q = 16 / (int)sizeof(T);  // values per 16 bytes
        constexpr int want = (PP % 32) / q * q;
        return 6 * NPS + ((want - 6 * NPS) % 32 + 32) % 32;
    }
    template <typename T>
    SESNT_HD static constexpr size_t stage_offset() { return ((sizeof(T) * SMEM_T + 127) / 128) * 128; }
    template <typename T>
    SESNT_HD static constexpr size_t smem(bool stage) {
        return stage ? stage_offset<T>() + sizeof(T) * (size_t)G * stage_stride<T>() + 16 : sizeof(T) * SMEM_T;
    }
    // k_element_cols2: slabs of (simulation 0, simulation 1) value pairs,
    // one unit every US2 pairs, congruent to PP modulo 16 so that thread t
    // finds the pair c of its unit in banks 2t and 2t + 1 (mod 32) for 4-byte
    // values (4t .. 4t + 3 for 8-byte values), as US does for single values.
    static constexpr int US2 = 9 * NP + ((PP - 9 * NP) % 16 + 16) % 16;
    template <typename T>
    SESNT_HD static constexpr size_t smem2() { return sizeof(T) * (4 * PP + 2 * (size_t)G * US2); }
};

// STAGE: thread 0 bulk-copies the block's stress range (G units of 6 x NPS
// values, contiguous and 16-byte aligned) into shared memory at the start,
// under one mbarrier with a bounded wait; the points read and write their
// stress there and thread 0 bulk-stores the range after the flux barrier.
// Without it each point loads its stress from global memory one point of the
// column ahead.
template <int N, typename T, bool ANISO, int MINB, bool STAGE>
__global__ void __launch_bounds__(ColCfg<N>::NT, MINB) k_element_cols(const StepArgs<T> a) {
    using C = ColCfg<N>;
    constexpr int P = C::P, PP = C::PP, NP = C::NP, G = C::G, NT = C::NT;
    constexpr int NPS = C::NPS;
    extern __shared__ __align__(128) unsigned char cols_smem_raw[];
    unsigned char *smem_raw = cols_smem_raw;
    T *sD = reinterpret_cast<T *>(smem_raw);  // [4][P*P]: Dx Dy Dz (scaled) | Dt
    const int t = threadIdx.x;
    const long long units = (long long)a.nel * a.S;
    const long long ufirst = (long long)blockIdx.x * G;
    const int nunits = (int)(units - ufirst < G ? units - ufirst : G);  // units of this block
    constexpr int SS = C::template stage_stride<T>();
    T *stage = reinterpret_cast<T *>(smem_raw + C::template stage_offset<T>());
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem_raw + C::template stage_offset<T>() + sizeof(T) * (size_t)G * SS);
    constexpr uint32_t unit_bytes = (uint32_t)(sizeof(T) * 6 * NPS);  // a multiple of 16
    bool issued = false;
    if constexpr (STAGE) {
        if (t == 0) {
            const uint32_t mb = tma_smem(mbar);
            tma_mbar_init(mb);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            if (!a.drop_completion && in_range((size_t)(ufirst + nunits) * 6 * NPS - 1, (size_t)units * 6 * NPS, a.err)) {
                tma_expect(mb, unit_bytes * (uint32_t)nunits);
                for (int u = 0; u < nunits; ++u)
                    tma_load_unit(stage + (size_t)u * SS, a.sig + (size_t)(ufirst + u) * 6 * NPS, unit_bytes, mb, a.piece);
                issued = true;
            }
        }
    }
    if (t == 0 && a.prefetch > 0 && ufirst + a.prefetch < units) {
        // L2 prefetch of the stress and material of the units a.prefetch
        // ahead: about those the block that next takes this slot will load
        const long long u1 = ufirst + a.prefetch, u2 = u1 + G < units ? u1 + G : units;
        l2_prefetch(a.sig + (size_t)u1 * 6 * NPS, sizeof(T) * (size_t)(u2 - u1) * 6 * NPS, a.sig,
                    a.sig + (size_t)units * 6 * NPS);
        const size_t e1 = (size_t)(u1 / a.S), e2 = (size_t)((u2 - 1) / a.S) + 1, nl = (size_t)a.nel * NP;
        const size_t bytes = sizeof(T) * (e2 - e1) * NP;
        l2_prefetch(a.lam + e1 * NP, bytes, a.lam, a.lam + nl);
        l2_prefetch(a.mu + e1 * NP, bytes, a.mu, a.mu + nl);
        if constexpr (ANISO) {
            l2_prefetch(a.A + e1 * NP, bytes, a.A, a.A + nl);
            l2_prefetch(a.B + e1 * NP, bytes, a.B, a.B + nl);
            l2_prefetch(a.C + e1 * NP, bytes, a.C, a.C + nl);
        }
    }
    for (int x = t; x < 4 * PP; x += NT) sD[x] = a.tabD[x];
    const int gl = t / PP;
    const int c = t - gl * PP;
    const int i = c % P, j = c / P;
    T *sv = sD + 4 * PP + (size_t)gl * C::US;   // this unit's [3][NP] velocity slab
    T *sx = sv + 3 * NP;                        // [3][NP] x fluxes (xx, xy, xz weighted)
    T *sy = sx + 3 * NP;                        // [3][NP] y fluxes
    const long long unit = ufirst + gl;
    const size_t nuni = (size_t)a.nuni, nloc = (size_t)a.nloc;
    int e = 0, s = 0, ex = 0, ey = 0, ez = 0;
    bool act = gl < G && unit < units;
    if (act) {
        e = (int)(unit / a.S);
        s = (int)(unit - (long long)e * a.S);
        ex = e % a.nx;
        ey = (e / a.nx) % a.ny;
        ez = e / (a.nx * a.ny);
        act = in_range(unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, N), nuni, a.err) &&
              in_range((size_t)e * NP + c + (size_t)PP * N, nloc, a.err) &&
              in_range((size_t)unit * 6 * NPS + 5 * NPS + c + (size_t)PP * N, (size_t)units * 6 * NPS, a.err);
    }
    const size_t kstep = (size_t)a.NXU * a.NYU;  // unique-index stride of k
    const size_t u0 = act ? unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, 0) : 0;
    const size_t l0 = (size_t)e * NP + c;        // element-local index of (i, j, 0)
    // this column's stress at k = 0: the staged copy or global memory
    T *sig = STAGE ? stage + (size_t)gl * SS + c : a.sig + (size_t)unit * 6 * NPS + c;
    T vc[3][P];  // this column's velocity
    if (act) {
        const T *vs = a.v + (size_t)s * 3 * nuni;
#pragma unroll
        for (int k = 0; k < P; ++k) {
            const size_t u = u0 + k * kstep;
            vc[0][k] = vs[u];
            vc[1][k] = vs[nuni + u];
            vc[2][k] = vs[2 * nuni + u];
        }
#pragma unroll
        for (int k = 0; k < P; ++k) {
            sv[c + PP * k] = vc[0][k];
            sv[NP + c + PP * k] = vc[1][k];
            sv[2 * NP + c + PP * k] = vc[2][k];
        }
    }
    // material and stress of point k = 0, in flight across the barrier
    T lam = 0, mu = 0, cA = 0, cB = 0, cC = 0, sg[6] = {0, 0, 0, 0, 0, 0};
    auto load_point = [&](int k, T &l, T &m_, T &A, T &B, T &Cc, T (&sgk)[6]) {
        const size_t li = l0 + (size_t)PP * k;
        l = ld_stream(a.lam + li);
        m_ = ld_stream(a.mu + li);
        if constexpr (ANISO) {
            A = ld_stream(a.A + li);
            B = ld_stream(a.B + li);
            Cc = ld_stream(a.C + li);
        }
        if constexpr (!STAGE) {
#pragma unroll
            for (int q = 0; q < 6; ++q) sgk[q] = ld_stream(sig + q * NPS + PP * k);
        }
    };
    if (act) load_point(0, lam, mu, cA, cB, cC, sg);
    __syncthreads();  // tables, velocity slabs and the mbarrier's initialisation
    bool landed = true;
    if constexpr (STAGE) landed = tma_try_wait(tma_smem(mbar), 0, a.wait_polls);
    const T *Dx = sD, *Dy = sD + PP, *Dt = sD + 3 * PP;  // z tables: a.tabz (compile-time indices)
    T dxi[P], dyj[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
        dxi[q] = Dx[q * P + i];
        dyj[q] = Dy[q * P + j];
    }
    T zf[3][P];  // z fluxes of this column: xz, yz, zz weighted (contracted along k)
    const T m0[6][1] = {{0}, {0}, {0}, {0}, {0}, {0}};
    // the column's metric values that do not change along k, loaded once
    PointMetric<T> pm{};
    if (act) {
        pm.ct = a.cot_t[ex * P + i];
        pm.isn = a.inv_sin[ex * P + i];
        pm.st = a.sin_t[ex * P + i];
        pm.px = a.px[ex * P + i];
        pm.py = a.py[ey * P + j];
        pm.wij = a.w[i] * a.w[j];
    }
#pragma unroll
    for (int k = 0; k < P; ++k) {
        T nlam = 0, nmu = 0, nA = 0, nB = 0, nC = 0, nsg[6] = {0, 0, 0, 0, 0, 0};
        if (k + 1 < P && act) load_point(k + 1, nlam, nmu, nA, nB, nC, nsg);
        if constexpr (STAGE) {
#pragma unroll
            for (int q = 0; q < 6; ++q) sg[q] = act && landed ? sig[q * NPS + PP * k] : T(0);
        }
        if (act && landed) {
            T ev[9];
#pragma unroll
            for (int x = 0; x < 9; ++x) ev[x] = 0;
            const T *row = sv + P * (j + P * k);  // x line (q, j, k)
            const T *col = sv + i + PP * k;       // y line (i, q, k)
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const T dx = dxi[q], dy = dyj[q], dz = a.tabz[0][q * P + k];
                ev[0] += row[q] * dx;
                ev[1] += row[NP + q] * dx;
                ev[2] += row[2 * NP + q] * dx;
                ev[3] += col[P * q] * dy;
                ev[4] += col[NP + P * q] * dy;
                ev[5] += col[2 * NP + P * q] * dy;
                ev[6] += vc[0][q] * dz;
                ev[7] += vc[1][q] * dz;
                ev[8] += vc[2][q] * dz;
            }
            T sn[6], gw[3];
            pm.ir = a.inv_r[ez * P + k];
            pm.rr = a.r[ez * P + k];
            pm.pz = a.pz[ez * P + k];
            pm.wk = a.w[k];
            point_stress<N, T, 0, ANISO, false, STAGE, true>(a, ev, vc[0][k], vc[1][k], vc[2][k], i, j, k, ex, ey, ez,
                                                             lam, mu, T(0), cA, cB, cC, sg, m0, sig + PP * k, nullptr,
                                                             NPS, nloc, nullptr, sn, gw, &pm);
            const int p = c + PP * k;
            sx[p] = sn[0] * gw[0];
            sx[NP + p] = sn[1] * gw[0];
            sx[2 * NP + p] = sn[2] * gw[0];
            sy[p] = sn[1] * gw[1];
            sy[NP + p] = sn[3] * gw[1];
            sy[2 * NP + p] = sn[4] * gw[1];
            zf[0][k] = sn[2] * gw[2];
            zf[1][k] = sn[4] * gw[2];
            zf[2][k] = sn[5] * gw[2];
        }
        lam = nlam;
        mu = nmu;
        cA = nA;
        cB = nB;
        cC = nC;
#pragma unroll
        for (int q = 0; q < 6; ++q) sg[q] = nsg[q];
    }
    // weak divergence of this column's points and their assembly
    auto column_divergence = [&]() {
        T dti[P], dtj[P];
#pragma unroll
        for (int q = 0; q < P; ++q) {
            dti[q] = Dt[i * P + q];
            dtj[q] = Dt[j * P + q];
        }
#pragma unroll
        for (int k = 0; k < P; ++k) {
            T fx = 0, fy = 0, fz = 0;
            const T *row = sx + P * (j + P * k);
            const T *col = sy + i + PP * k;
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const T di = dti[q], dj = dtj[q], dk = a.tabz[1][k * P + q];
                fx += zf[0][q] * dk + col[P * q] * dj + row[q] * di;
                fy += zf[1][q] * dk + col[NP + P * q] * dj + row[NP + q] * di;
                fz += zf[2][q] * dk + col[2 * NP + P * q] * dj + row[2 * NP + q] * di;
            }
            const size_t u = u0 + k * kstep;
            add_force(a, s, u, fx, fy, fz);
        }
    };
    // updated stress in the stage: visible to the bulk-copy engine after the barrier
    if constexpr (STAGE) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const bool ok = __syncthreads_and(landed) != 0;  // x and y flux slabs
    if constexpr (STAGE) {
        if (t == 0) {
            if (ok) {
                for (int u = 0; u < nunits; ++u)
                    tma_store(a.sig + (size_t)(ufirst + u) * 6 * NPS, tma_smem(stage + (size_t)u * SS), unit_bytes);
                tma_commit();
            } else {
                atomicExch(a.err, 1);
                // the copy may still be in flight: one more bounded wait
                // before the block's shared memory is released
                if (issued) tma_try_wait(tma_smem(mbar), 0, a.wait_polls);
            }
        }
    }
    if (act && ok) column_divergence();
    if constexpr (STAGE)
        if (ok && t == 0) tma_wait_read<0>();  // the store has read the stage before it is released
}


template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
    using type = float2;
};
template <>
struct Vec2<double> {
    using type = double2;
};

// Two simulations per column thread (k_element_cols2), for even elastic
// batches. A unit is an element and a pair of consecutive simulations
// (2p, 2p + 1), whose stress units are adjacent in the element-major state.
// The slabs hold (simulation 2p, simulation 2p + 1) value pairs, so one
// 8-byte shared load (16 bytes in FP64) feeds both simulations' line
// contractions, and the point's derivative-table registers, metric, taper,
// material and index arithmetic serve both, as in k_element_pair. Each
// thread keeps both simulations' column velocities and z fluxes in
// registers. Per point and simulation the arithmetic and its order are
// those of k_element_pair.
template <int N, typename T, bool ANISO, int MINB>
__global__ void __launch_bounds__(ColCfg<N>::NT, MINB) k_element_cols2(const StepArgs<T> a) {
    using C = ColCfg<N>;
    using V = typename Vec2<T>::type;
    constexpr int P = C::P, PP = C::PP, NP = C::NP, G = C::G, NT = C::NT, NPS = C::NPS, US = C::US2;
    extern __shared__ __align__(128) unsigned char cols_smem_raw[];
    T *sD = reinterpret_cast<T *>(cols_smem_raw);  // [4][P*P]: Dx Dy Dz (scaled) | Dt
    V *slab = reinterpret_cast<V *>(sD + 4 * PP);  // 16-byte aligned: 4 * PP values of T
    const int t = threadIdx.x;
    const int S2 = a.S / 2;
    const long long units = (long long)a.nel * S2;
    const long long ufirst = (long long)blockIdx.x * G;
    const size_t ustate = (size_t)6 * NPS;                 // values of one simulation's stress unit
    const size_t nstate = (size_t)a.nel * a.S * ustate;    // the whole stress array
    if (t == 0 && a.prefetch > 0 && ufirst + a.prefetch < units) {
        // L2 prefetch of the stress and material of the units a.prefetch ahead
        const long long u1 = ufirst + a.prefetch, u2 = u1 + G < units ? u1 + G : units;
        l2_prefetch(a.sig + (size_t)(2 * u1) * ustate, sizeof(T) * (size_t)(2 * (u2 - u1)) * ustate, a.sig,
                    a.sig + nstate);
        const size_t e1 = (size_t)(u1 / S2), e2 = (size_t)((u2 - 1) / S2) + 1, nl = (size_t)a.nel * NP;
        const size_t bytes = sizeof(T) * (e2 - e1) * NP;
        l2_prefetch(a.lam + e1 * NP, bytes, a.lam, a.lam + nl);
        l2_prefetch(a.mu + e1 * NP, bytes, a.mu, a.mu + nl);
        if constexpr (ANISO) {
            l2_prefetch(a.A + e1 * NP, bytes, a.A, a.A + nl);
            l2_prefetch(a.B + e1 * NP, bytes, a.B, a.B + nl);
            l2_prefetch(a.C + e1 * NP, bytes, a.C, a.C + nl);
        }
    }
    for (int x = t; x < 4 * PP; x += NT) sD[x] = a.tabD[x];
    const int gl = t / PP;
    const int c = t - gl * PP;
    const int i = c % P, j = c / P;
    V *sv = slab + (size_t)gl * US;  // this unit's [3][NP] velocity pairs
    V *sx = sv + 3 * NP;             // [3][NP] x fluxes (xx, xy, xz weighted)
    V *sy = sx + 3 * NP;             // [3][NP] y fluxes (xy, yy, yz weighted)
    const long long unit = ufirst + gl;
    const size_t nuni = (size_t)a.nuni, nloc = (size_t)a.nloc;
    int e = 0, s0 = 0, ex = 0, ey = 0, ez = 0;
    bool act = gl < G && unit < units;
    if (act) {
        e = (int)(unit / S2);
        s0 = 2 * (int)(unit - (long long)e * S2);
        ex = e % a.nx;
        ey = (e / a.nx) % a.ny;
        ez = e / (a.nx * a.ny);
        act = in_range(unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, N), nuni, a.err) &&
              in_range((size_t)e * NP + c + (size_t)PP * N, nloc, a.err) &&
              in_range((size_t)(s0 + 1), (size_t)a.S, a.err) &&
              in_range((size_t)(2 * unit + 1) * ustate + 5 * NPS + c + (size_t)PP * N, nstate, a.err);
    }
    const size_t kstep = (size_t)a.NXU * a.NYU;  // unique-index stride of k
    const size_t u0 = act ? unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, 0) : 0;
    const size_t l0 = (size_t)e * NP + c;        // element-local index of (i, j, 0)
    const size_t soff = act ? (size_t)(2 * unit) * ustate + c : 0;
    T *sig0 = a.sig + soff, *sig1 = sig0 + ustate;  // this column's stress at k = 0
    T vc[2][3][P];  // the column's velocity, both simulations
    if (act) {
        const T *va = a.v + (size_t)s0 * 3 * nuni, *vb = va + 3 * nuni;
#pragma unroll
        for (int k = 0; k < P; ++k) {
            const size_t u = u0 + k * kstep;
            vc[0][0][k] = va[u];
            vc[0][1][k] = va[nuni + u];
            vc[0][2][k] = va[2 * nuni + u];
            vc[1][0][k] = vb[u];
            vc[1][1][k] = vb[nuni + u];
            vc[1][2][k] = vb[2 * nuni + u];
        }
#pragma unroll
        for (int k = 0; k < P; ++k) {
#pragma unroll
            for (int q = 0; q < 3; ++q) sv[q * NP + c + PP * k] = V{vc[0][q][k], vc[1][q][k]};
        }
    }
    // material and stress of point k = 0, in flight across the barrier
    T lam = 0, mu = 0, cA = 0, cB = 0, cC = 0, sg[2][6] = {{0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0}};
    auto load_point = [&](int k, T &l, T &m_, T &A, T &B, T &Cc, T (&sgk)[2][6]) {
        const size_t li = l0 + (size_t)PP * k;
        l = ld_stream(a.lam + li);
        m_ = ld_stream(a.mu + li);
        if constexpr (ANISO) {
            A = ld_stream(a.A + li);
            B = ld_stream(a.B + li);
            Cc = ld_stream(a.C + li);
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            sgk[0][q] = ld_stream(sig0 + q * NPS + PP * k);
            sgk[1][q] = ld_stream(sig1 + q * NPS + PP * k);
        }
    };
    if (act) load_point(0, lam, mu, cA, cB, cC, sg);
    __syncthreads();  // tables and velocity slabs
    const T *Dx = sD, *Dy = sD + PP, *Dt = sD + 3 * PP;  // z tables: a.tabz (compile-time indices)
    T dxi[P], dyj[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
        dxi[q] = Dx[q * P + i];
        dyj[q] = Dy[q * P + j];
    }
    T zf[2][3][P];  // z fluxes of the column (xz, yz, zz weighted), both simulations
    const T m0[6][1] = {{0}, {0}, {0}, {0}, {0}, {0}};
    // the column's metric values that do not change along k, loaded once
    T ct = 0, isn = 0, st = 0, pxv = 0, pyv = 0, wij = 0;
    if (act) {
        ct = a.cot_t[ex * P + i];
        isn = a.inv_sin[ex * P + i];
        st = a.sin_t[ex * P + i];
        pxv = a.px[ex * P + i];
        pyv = a.py[ey * P + j];
        wij = a.w[i] * a.w[j];
    }
#pragma unroll
    for (int k = 0; k < P; ++k) {
        T nlam = 0, nmu = 0, nA = 0, nB = 0, nC = 0, nsg[2][6] = {{0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0}};
        if (k + 1 < P && act) load_point(k + 1, nlam, nmu, nA, nB, nC, nsg);
        if (act) {
            T e0[9], e1[9];
#pragma unroll
            for (int x = 0; x < 9; ++x) e0[x] = e1[x] = 0;
            const V *row = sv + P * (j + P * k);  // x line (q, j, k)
            const V *col = sv + i + PP * k;       // y line (i, q, k)
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const T dx = dxi[q], dy = dyj[q], dz = a.tabz[0][q * P + k];
                const V rx = row[q], ry = row[NP + q], rz = row[2 * NP + q];
                const V cx = col[P * q], cy = col[NP + P * q], cz = col[2 * NP + P * q];
                e0[0] += rx.x * dx;
                e0[1] += ry.x * dx;
                e0[2] += rz.x * dx;
                e0[3] += cx.x * dy;
                e0[4] += cy.x * dy;
                e0[5] += cz.x * dy;
                e0[6] += vc[0][0][q] * dz;
                e0[7] += vc[0][1][q] * dz;
                e0[8] += vc[0][2][q] * dz;
                e1[0] += rx.y * dx;
                e1[1] += ry.y * dx;
                e1[2] += rz.y * dx;
                e1[3] += cx.y * dy;
                e1[4] += cy.y * dy;
                e1[5] += cz.y * dy;
                e1[6] += vc[1][0][q] * dz;
                e1[7] += vc[1][1][q] * dz;
                e1[8] += vc[1][2][q] * dz;
            }
            const T ir = a.inv_r[ez * P + k], irs = ir * isn;
            T g0[9], g1[9];
            complete_gradient_m<T>(e0, vc[0][0][k], vc[0][1][k], vc[0][2][k], ir, ct, irs, g0);
            complete_gradient_m<T>(e1, vc[1][0][k], vc[1][1][k], vc[1][2][k], ir, ct, irs, g1);
            const T tp = taper_value(pxv, pyv, a.pz[ez * P + k], a.inv_alpha);
            const T rr = a.r[ez * P + k];
            const T rs = rr * st;
            const T W = wij * a.w[k];
            const T gx = W * rs * a.c1, gy = W * rr * a.c2, gz = W * (rr * rs) * a.c3;
            T sn[2][6];  // integrated stress before the taper: xx xy xz yy yz zz
            auto update = [&](const T(&gg)[9], const T(&sgv)[6], T *sig, T(&o)[6]) {
                const T exx = gg[kDuXX], eyy = gg[kDuYY], ezz = gg[kDuZZ];
                const T exy = (gg[kDuXY] + gg[kDuYX]) * T(0.5);
                const T exz = (gg[kDuXZ] + gg[kDuZX]) * T(0.5);
                const T eyz = (gg[kDuYZ] + gg[kDuZY]) * T(0.5);
                T rxx, ryy, rzz, rxy, rxz, ryz;
                stress_rates<T, 0, ANISO>(exx, eyy, ezz, exy, exz, eyz, lam, mu, T(0), cA, cB, cC, m0, rxx, ryy,
                                          rzz, rxy, rxz, ryz);
                o[0] = sgv[0] + a.dt * rxx;
                o[1] = sgv[1] + a.dt * rxy;
                o[2] = sgv[2] + a.dt * rxz;
                o[3] = sgv[3] + a.dt * ryy;
                o[4] = sgv[4] + a.dt * ryz;
                o[5] = sgv[5] + a.dt * rzz;
#pragma unroll
                for (int q = 0; q < 6; ++q) st_stream(sig + q * NPS, o[q] * tp);
            };
            update(g0, sg[0], sig0 + PP * k, sn[0]);
            update(g1, sg[1], sig1 + PP * k, sn[1]);
            const int p = c + PP * k;
            sx[p] = V{sn[0][0] * gx, sn[1][0] * gx};
            sx[NP + p] = V{sn[0][1] * gx, sn[1][1] * gx};
            sx[2 * NP + p] = V{sn[0][2] * gx, sn[1][2] * gx};
            sy[p] = V{sn[0][1] * gy, sn[1][1] * gy};
            sy[NP + p] = V{sn[0][3] * gy, sn[1][3] * gy};
            sy[2 * NP + p] = V{sn[0][4] * gy, sn[1][4] * gy};
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                zf[s][0][k] = sn[s][2] * gz;
                zf[s][1][k] = sn[s][4] * gz;
                zf[s][2][k] = sn[s][5] * gz;
            }
        }
        lam = nlam;
        mu = nmu;
        cA = nA;
        cB = nB;
        cC = nC;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            sg[0][q] = nsg[0][q];
            sg[1][q] = nsg[1][q];
        }
    }
    __syncthreads();  // x and y flux slabs
    if (!act) return;
    // weak divergence of the column's points, both simulations, and their assembly
    T dti[P], dtj[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
        dti[q] = Dt[i * P + q];
        dtj[q] = Dt[j * P + q];
    }
#pragma unroll
    for (int k = 0; k < P; ++k) {
        T f[2][3] = {{0, 0, 0}, {0, 0, 0}};
        const V *row = sx + P * (j + P * k);
        const V *col = sy + i + PP * k;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const T di = dti[q], dj = dtj[q], dk = a.tabz[1][k * P + q];
            const V r0 = row[q], r1 = row[NP + q], r2 = row[2 * NP + q];
            const V c0 = col[P * q], c1 = col[NP + P * q], c2 = col[2 * NP + P * q];
            f[0][0] += zf[0][0][q] * dk + c0.x * dj + r0.x * di;
            f[0][1] += zf[0][1][q] * dk + c1.x * dj + r1.x * di;
            f[0][2] += zf[0][2][q] * dk + c2.x * dj + r2.x * di;
            f[1][0] += zf[1][0][q] * dk + c0.y * dj + r0.y * di;
            f[1][1] += zf[1][1][q] * dk + c1.y * dj + r1.y * di;
            f[1][2] += zf[1][2][q] * dk + c2.y * dj + r2.y * di;
        }
        const size_t u = u0 + k * kstep;
        add_force(a, s0, u, f[0][0], f[0][1], f[0][2]);
        add_force(a, s0 + 1, u, f[1][0], f[1][1], f[1][2]);
    }
}

// Resident blocks per SM the paired column kernel is sized for (FP32; FP64
// uses 1). At degree 4 its 45 KB of slabs allow at most 4 blocks per SM; at
// 2 blocks (175 registers in FP32) the kernel needs no cap on registers.
constexpr int kCols2Minb[] = {4, 3, 2, 2};

template <int N, typename T, bool ANISO, int MINB>
int launch_element_cols2_m(const StepArgs<T> &a, void *stream) {
    using C = ColCfg<N>;
    if (a.S < 2 || a.S % 2 != 0) return 1;
    const long long units = (long long)a.nel * (a.S / 2);
    const size_t smem = C::template smem2<T>();
    if (smem > kMaxSmemPerBlock) return 1;
    k_element_cols2<N, T, ANISO, MINB><<<(unsigned)((units + C::G - 1) / C::G), C::NT, smem, (cudaStream_t)stream>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// minb_idx selects kCols2Minb[] (FP32); returns 1 if this configuration has
// no paired column kernel (the caller falls back).
template <int N, typename T, bool ANISO>
int launch_element_cols2(const StepArgs<T> &a, int minb_idx, void *stream) {
    if constexpr (sizeof(T) == 8) {
        return launch_element_cols2_m<N, T, ANISO, 1>(a, stream);
    } else {
        switch (minb_idx) {
            case 0: return launch_element_cols2_m<N, T, ANISO, kCols2Minb[0]>(a, stream);
            case 1: return launch_element_cols2_m<N, T, ANISO, kCols2Minb[1]>(a, stream);
            case 2: return launch_element_cols2_m<N, T, ANISO, kCols2Minb[2]>(a, stream);
            default: return launch_element_cols2_m<N, T, ANISO, kCols2Minb[3]>(a, stream);
        }
    }
}

template <int N, typename T, bool ANISO, int MINB>
int prepare_element_cols2_m() {
    const size_t smem = ColCfg<N>::template smem2<T>();
    if (smem <= 48 * 1024 || smem > kMaxSmemPerBlock) return 0;
    return cudaFuncSetAttribute(k_element_cols2<N, T, ANISO, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem) == cudaSuccess
               ? 0
               : -1;
}

// Resident blocks per SM the column kernel is sized for (FP32); FP64 uses 1
// (as k_element). Selected per grid by the tuner among the instantiated
// values.
constexpr int kColsMinb[] = {4, 5, 6, 8};

template <int N, typename T, bool ANISO, int MINB, bool STAGE>
int launch_element_cols_m(const StepArgs<T> &a, void *stream) {
    using C = ColCfg<N>;
    const long long units = (long long)a.nel * a.S;
    const size_t smem = C::template smem<T>(STAGE);
    if (smem > kMaxSmemPerBlock) return 1;
    k_element_cols<N, T, ANISO, MINB, STAGE>
        <<<(unsigned)((units + C::G - 1) / C::G), C::NT, smem, (cudaStream_t)stream>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// minb_idx selects kColsMinb[] (FP32); returns 1 if this configuration has
// no column kernel (the caller falls back).
template <int N, typename T, bool ANISO, bool STAGE>
int launch_element_cols(const StepArgs<T> &a, int minb_idx, void *stream) {
    if constexpr (sizeof(T) == 8) {
        return launch_element_cols_m<N, T, ANISO, 1, STAGE>(a, stream);
    } else {
        switch (minb_idx) {
            case 0: return launch_element_cols_m<N, T, ANISO, kColsMinb[0], STAGE>(a, stream);
            case 1: return launch_element_cols_m<N, T, ANISO, kColsMinb[1], STAGE>(a, stream);
            case 2: return launch_element_cols_m<N, T, ANISO, kColsMinb[2], STAGE>(a, stream);
            default: return launch_element_cols_m<N, T, ANISO, kColsMinb[3], STAGE>(a, stream);
        }
    }
}

template <int N, typename T, bool ANISO, int MINB>
int prepare_element_cols_m() {
    for (bool stage : {false, true}) {
        const size_t smem = ColCfg<N>::template smem<T>(stage);
        if (smem <= 48 * 1024 || smem > kMaxSmemPerBlock) continue;
        auto f = stage ? k_element_cols<N, T, ANISO, MINB, true> : k_element_cols<N, T, ANISO, MINB, false>;
        if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    }
    return 0;
}

template <int N, typename T, bool ANISO>
int prepare_element_cols() {
    if constexpr (sizeof(T) == 8)
        return prepare_element_cols_m<N, T, ANISO, 1>() || prepare_element_cols2_m<N, T, ANISO, 1>() ? -1 : 0;
    else
        return prepare_element_cols_m<N, T, ANISO, kColsMinb[0]>() || prepare_element_cols_m<N, T, ANISO, kColsMinb[1]>() ||
                       prepare_element_cols_m<N, T, ANISO, kColsMinb[2]>() || prepare_element_cols_m<N, T, ANISO, kColsMinb[3]>() ||
                       prepare_element_cols2_m<N, T, ANISO, kCols2Minb[0]>() ||
                       prepare_element_cols2_m<N, T, ANISO, kCols2Minb[1]>() ||
                       prepare_element_cols2_m<N, T, ANISO, kCols2Minb[2]>() ||
                       prepare_element_cols2_m<N, T, ANISO, kCols2Minb[3]>()
                   ? -1
                   : 0;
}

}  // namespace sesnt
