// Persistent element kernel fed by the tensor memory accelerator (bulk
// copies). Each element's stress and memory variables are one contiguous,
// 16-byte aligned unit of the element-blocked state (StateLayout), so one
// cp.async.bulk moves a whole element into shared memory,
// tracked by an mbarrier with a transaction count, NSTAGE-1 elements ahead of
// the one being computed. The updated state is written back into the same
// shared-memory stage and stored with one bulk copy
// (cp.async.bulk ... bulk_group), so the streaming traffic costs no per-thread
// load/store instructions and no registers. Velocity gathers, material and
// the contractions are as in k_element.
//
// Per block (one element at a time, thread p owns point p):
//   wait stage k%NSTAGE -> velocity slab -> point update (state read from and
//   written to the stage) -> bulk store of the stage -> bulk load of element
//   k+NSTAGE-1 into the stage element k-1 used (after its store has read it)
//   -> weak divergence and atomic assembly.
// Every mbarrier wait is bounded (StepArgs::wait_polls); on expiry the block
// sets the error word and leaves the loop with all its threads.
#pragma once

namespace sesnt {

__device__ __forceinline__ uint32_t tma_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tma_mbar_init(uint32_t mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
}

// Arrive once and add `bytes` to the transaction count of this phase.
__device__ __forceinline__ void tma_expect(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tma_store(void *dst, uint32_t src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Wait until at most NPEND committed bulk groups of this thread still read
// shared memory (their source may then be overwritten).
template <int NPEND>
__device__ __forceinline__ void tma_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(NPEND) : "memory");
}

// Wait until every committed bulk group of this thread has completed.
__device__ __forceinline__ void tma_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ bool tma_try_wait(uint32_t mbar, uint32_t parity, int polls) {
    uint32_t done = 0;
    for (int it = 0; it < polls && !done; ++it)
        asm volatile(
            "{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p;}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
    return done != 0;
}

// The same wait polled by lane 0 of each warp only: the outcome goes to the
// other lanes by shuffle, and __syncwarp orders their later reads of the
// landed data after lane 0's acquiring wait. Every thread of the warp must
// call it. Where all lanes poll, each poll is a shared-memory operation per
// lane.
__device__ __forceinline__ bool tma_try_wait_warp(uint32_t mbar, uint32_t parity, int polls) {
    bool done = false;
    if ((threadIdx.x & 31) == 0) done = tma_try_wait(mbar, parity, polls);
    done = __shfl_sync(0xffffffffu, done ? 1 : 0, 0) != 0;
    __syncwarp();
    return done;
}

// A hint that brings [p, p + bytes) of global memory into L2 (bulk
// prefetch; no completion, no effect on results). The range is narrowed to
// 16-byte boundaries inside [lo, hi), the buffer it belongs to.
__device__ __forceinline__ void l2_prefetch(const void *p, size_t bytes, const void *lo, const void *hi) {
    uintptr_t a = (uintptr_t)p, b = a + bytes;
    const uintptr_t l = ((uintptr_t)lo + 15) & ~(uintptr_t)15, h = (uintptr_t)hi & ~(uintptr_t)15;
    a = a < l ? l : (a & ~(uintptr_t)15);
    b = b > h ? h : ((b + 15) & ~(uintptr_t)15);
    for (; a < b; a += 16384) {  // in pieces of at most 16 KB
        const uint32_t n = (uint32_t)(b - a < 16384 ? b - a : 16384);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"(n) : "memory");
    }
}

// Bulk copies of one state unit are issued in pieces of at most `piece`
// bytes (StepArgs::piece, a multiple of 16; 0: one copy per unit), so every
// piece starts 16-byte aligned inside the 16-byte aligned unit. The 33 KB
// units of degree 6 load 2.2% faster in 8 KB pieces than as one copy; degree
// 4 (12 KB) is the same either way. The tuner sweeps the size per grid.
template <typename T>
__device__ __forceinline__ void tma_load_unit(T *dst, const T *src, uint32_t bytes, uint32_t mbar, int piece) {
    const uint32_t pc = piece > 0 ? ((uint32_t)piece & ~15u) : bytes;
    const uint32_t step = pc > 0 ? pc : bytes;
    for (uint32_t off = 0; off < bytes; off += step)
        tma_load(tma_smem(reinterpret_cast<unsigned char *>(dst) + off), reinterpret_cast<const unsigned char *>(src) + off,
                 bytes - off < step ? bytes - off : step, mbar);
}

#ifndef SESNT_TMA_STAGES
#define SESNT_TMA_STAGES 3
#endif

template <int N, typename T, int NSLS>
struct TmaCfg {
    static constexpr int P = N + 1, NP = P * P * P, NPS = StateLayout<NP, NSLS>::CS;
    static constexpr int NT = ((NP + 31) / 32) * 32;
    static constexpr int MS = NSLS > 0 ? NSLS : 1;
    static constexpr int NSTAGE = SESNT_TMA_STAGES;
    static constexpr size_t UNIT = StateLayout<NP, NSLS>::UNIT;
    static constexpr uint32_t STAGE_BYTES = (uint32_t)(UNIT * sizeof(T));  // one unit, a multiple of 16
    // stages, then sD [4][P*P], sv [3][NP], sf [9][NP], then the mbarriers
    static constexpr size_t SMALL = sizeof(T) * (4 * P * P + 12 * NP);
    static constexpr size_t SMEM = NSTAGE * (size_t)STAGE_BYTES + ((SMALL + 15) / 16) * 16 + 8 * NSTAGE;
    // resident blocks the register allocation is sized for: as many as the
    // shared memory allows, at most 8 and at most 2048 threads
    static constexpr int MINB_RAW = (int)((227 * 1024) / SMEM);
    static constexpr int MINB_CAP = (2048 / NT) < 8 ? (2048 / NT) : 8;
    static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > MINB_CAP ? MINB_CAP : MINB_RAW);
};

template <int N, typename T, int NSLS, bool ANISO>
__global__ void __launch_bounds__(TmaCfg<N, T, NSLS>::NT, TmaCfg<N, T, NSLS>::MINB) k_element_tma(const StepArgs<T> a) {
    using C = TmaCfg<N, T, NSLS>;
    constexpr int P = C::P, NP = C::NP, NPS = C::NPS, NT = C::NT, MS = C::MS, NSTAGE = C::NSTAGE;
    extern __shared__ __align__(128) unsigned char tma_smem_raw[];
    unsigned char *stage0 = tma_smem_raw;
    T *sD = reinterpret_cast<T *>(tma_smem_raw + NSTAGE * (size_t)C::STAGE_BYTES);
    T *sv = sD + 4 * P * P;
    T *sf = sv + 3 * NP;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(tma_smem_raw + NSTAGE * (size_t)C::STAGE_BYTES +
                                                  ((C::SMALL + 15) / 16) * 16);

    const int t = threadIdx.x;
    const int S = a.S;
    const long long units = (long long)a.nel * S;
    const long long first = blockIdx.x, stride = gridDim.x;
    const int count = first < units ? (int)((units - 1 - first) / stride + 1) : 0;
    if (count == 0) return;
    const size_t nuni = (size_t)a.nuni, nloc = (size_t)a.nloc;

    for (int x = t; x < 4 * P * P; x += NT) sD[x] = a.tabD[x];
    if (t == 0) {
        for (int b = 0; b < NSTAGE; ++b) tma_mbar_init(tma_smem(mbar + b));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // bulk loads of unit k (this block's k-th element-simulation) into stage k % NSTAGE
    auto issue_load = [&](int k) {
        if (a.drop_completion) return;  // failure-detection test: the stage never lands
        const long long g = first + (long long)k * stride;
        const int b = k % NSTAGE;
        unsigned char *st = stage0 + (size_t)b * C::STAGE_BYTES;
        const uint32_t mb = tma_smem(mbar + b);
        tma_expect(mb, C::STAGE_BYTES);
        tma_load_unit(reinterpret_cast<T *>(st), a.sig + (size_t)g * C::UNIT, C::STAGE_BYTES, mb, a.piece);
    };
    if (t == 0)
        for (int k = 0; k < NSTAGE - 1 && k < count; ++k) issue_load(k);

    const int p = t;
    const bool act = p < NP;
    const int i = p % P, j = (p / P) % P, k3 = p / (P * P);
    // velocity and material of unit k, gathered ahead into registers
    T nv[3] = {0, 0, 0}, nlam = 0, nmu = 0, ntau = 0, nA = 0, nB = 0, nC = 0;
    auto gather = [&](int k) {
        if (!act || k >= count) return;
        const long long g = first + (long long)k * stride;
        const int e = (int)(g / S), s = (int)(g % S);
        const int ex = e % a.nx, ey = (e / a.nx) % a.ny, ez = e / (a.nx * a.ny);
        const size_t u = unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k3);
        if (!in_range(u, nuni, a.err) || !in_range((size_t)e * NP + p, nloc, a.err)) return;
        const T *vs = a.v + (size_t)s * 3 * nuni;
        nv[0] = vs[u];
        nv[1] = vs[nuni + u];
        nv[2] = vs[2 * nuni + u];
        const size_t li = (size_t)e * NP + p;
        nlam = a.lam[li];
        nmu = a.mu[li];
        if constexpr (NSLS > 0) ntau = a.tau[li];
        if constexpr (ANISO) {
            nA = a.A[li];
            nB = a.B[li];
            nC = a.C[li];
        }
    };
    gather(0);

    bool ok = true;
    int kfail = count;
    for (int k = 0; k < count; ++k) {
        const long long g = first + (long long)k * stride;
        const int e = (int)(g / S), s = (int)(g % S);
        const int ex = e % a.nx, ey = (e / a.nx) % a.ny, ez = e / (a.nx * a.ny);
        const int b = k % NSTAGE;
        T *st = reinterpret_cast<T *>(stage0 + (size_t)b * C::STAGE_BYTES);
        const T vx = nv[0], vy = nv[1], vz = nv[2], lam = nlam, mu = nmu, tau = ntau, cA = nA, cB = nB, cC = nC;
        if (act) {
            sv[p] = vx;
            sv[NP + p] = vy;
            sv[2 * NP + p] = vz;
        }
        // the stage of unit k has landed (block-uniform outcome)
        ok = __syncthreads_and(tma_try_wait(tma_smem(mbar + b), (uint32_t)((k / NSTAGE) & 1), a.wait_polls)) != 0;
        if (!ok) {
            kfail = k;
            break;
        }
        gather(k + 1);  // next unit's velocity and material, in flight during this one
        size_t u = 0;
        if (act) {
            u = unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k3);
            T sg[6], m[6][MS];
#pragma unroll
            for (int c = 0; c < 6; ++c) sg[c] = st[c * NPS + p];
            if constexpr (NSLS > 0) {
#pragma unroll
                for (int c = 0; c < 6; ++c)
#pragma unroll
                    for (int q = 0; q < NSLS; ++q) m[c][q] = st[6 * NPS + (c * NSLS + q) * NPS + p];
            }
            T ev[9];
            strain_contract<N, T>(sD, sv, sv + NP, sv + 2 * NP, i, j, k3, ev);
            point_update<N, T, NSLS, ANISO, false, true>(a, ev, vx, vy, vz, p, i, j, k3, ex, ey, ez, lam, mu, tau,
                                                         cA, cB, cC, sg, m, st + p, st + 6 * NPS + p, NPS, nloc, sf,
                                                         nullptr);
        }
        // state written back into the stage: hand it to the bulk-copy engine
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (t == 0) {
            tma_store(a.sig + (size_t)g * C::UNIT, tma_smem(st), C::STAGE_BYTES);
            tma_commit();
            if (k + NSTAGE - 1 < count) {
                // stage (k-1) % NSTAGE: its store (the group before this one) must have read it
                tma_wait_read<1>();
                issue_load(k + NSTAGE - 1);
            }
        }
        if (act) {
            T fx = 0, fy = 0, fz = 0;
            point_divergence<N, T>(sD + 3 * P * P, sf, i, j, k3, fx, fy, fz);
            add_force(a, s, u, fx, fy, fz);
        }
        __syncthreads();  // sv and sf are rewritten by the next unit
    }
    if (!ok && t == 0) atomicExch(a.err, 1);
    if (t == 0) tma_wait_all();  // stores complete; loads of a failed run are waited for below
    if (!ok) {
        // the loads issued for units kfail .. kfail+NSTAGE-2 may still be in
        // flight: one more bounded wait each before the shared memory is released
        for (int k = kfail; k < count && k < kfail + NSTAGE - 1; ++k)
            tma_try_wait(tma_smem(mbar + (k % NSTAGE)), (uint32_t)((k / NSTAGE) & 1), a.wait_polls);
    }
}

// One element per block with its stress and memory variables staged by bulk
// copy (k_element_stage), the default SLS step for degrees with one element
// per block (4-7): thread 0 starts the copy of the element's state unit
// (stress and memory variables, one contiguous range, in 8 KB pieces)
// before the velocity gather, so it travels during the gather, the staging
// barrier and the line contractions, and the state costs no per-thread load
// instructions or registers. The updated state goes back
// into the stage and out by bulk store (STORE), or from registers as in
// k_element (the default for degree 6). Measured on 3-SLS FP32 grids of 6-7 M points
// against k_element: 3.2/4.1/10.1/10.8% faster for degrees 4/5/6/7 (degree
// 6: 9.4% with the bulk store); FP64 unchanged. On elastic grids (one 3 KB
// chunk per element) it was 1-3% slower for degrees 4-6, so they keep
// k_element.
template <int N, typename T, int NSLS>
struct StageCfg {
    static constexpr int P = N + 1, NP = P * P * P, NPS = StateLayout<NP, NSLS>::CS;
    static constexpr int NT = ((NP + 31) / 32) * 32;
    static constexpr size_t UNIT = StateLayout<NP, NSLS>::UNIT;
    static constexpr uint32_t STAGE_BYTES = (uint32_t)(UNIT * sizeof(T));  // one unit, a multiple of 16
    static constexpr size_t SMALL = sizeof(T) * (4 * P * P + 12 * NP);
    static constexpr size_t SMEM = STAGE_BYTES + ((SMALL + 15) / 16) * 16 + 8;
    static constexpr bool STORE_DEFAULT = N != 6;
#ifndef SESNT_MINB_STAGE
#define SESNT_MINB_STAGE 8
#endif
    static constexpr int MINB = sizeof(T) == 4 ? (NT <= 128 ? SESNT_MINB_STAGE : ElemCfg<N>::MINB) : 1;
};

// KS: compensated stress integration (SESNT_FLAG_KAHAN_STRESS), register
// stores only; each thread loads and stores its point's compensation terms.
template <int N, typename T, int NSLS, bool ANISO, bool STORE, bool KS = false>
__global__ void __launch_bounds__(StageCfg<N, T, NSLS>::NT, StageCfg<N, T, NSLS>::MINB) k_element_stage(const StepArgs<T> a) {
    static_assert(!(STORE && KS), "compensated stress integration stores from registers");
    using C = StageCfg<N, T, NSLS>;
    constexpr int P = C::P, NP = C::NP, NPS = C::NPS, NT = C::NT, MS = NSLS > 0 ? NSLS : 1;
    extern __shared__ __align__(128) unsigned char stage_smem_raw[];
    T *st = reinterpret_cast<T *>(stage_smem_raw);  // one unit (StateLayout)
    T *sD = reinterpret_cast<T *>(stage_smem_raw + C::STAGE_BYTES);
    T *sv = sD + 4 * P * P;
    T *sf = sv + 3 * NP;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(stage_smem_raw + C::STAGE_BYTES + ((C::SMALL + 15) / 16) * 16);

    const int S = a.S;
    const int s = blockIdx.x % S;
    const int e = blockIdx.x / S;
    const int t = threadIdx.x;
    const size_t sb = (size_t)e * S + s;
    const bool blk = e < a.nel && in_range(sb * C::UNIT + C::UNIT - 1, (size_t)a.nel * S * C::UNIT, a.err);
    if (!blk) return;
    bool issued = false;
    if (t == 0) {
        const uint32_t mb = tma_smem(mbar);
        tma_mbar_init(mb);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (!a.drop_completion) {  // failure-detection test: the stage never lands
            tma_expect(mb, C::STAGE_BYTES);
            tma_load_unit(st, a.sig + sb * C::UNIT, C::STAGE_BYTES, mb, a.piece);
            issued = true;
        }
        // L2 prefetch of the state and material of the unit a.prefetch ahead:
        // about the unit the block that next takes this slot will load
        const size_t units = (size_t)a.nel * S, ahead = sb + (size_t)a.prefetch;
        if (a.prefetch > 0 && ahead < units) {
            l2_prefetch(a.sig + ahead * C::UNIT, C::STAGE_BYTES, a.sig, a.sig + units * C::UNIT);
            if (ahead % S == 0) {  // the material once per element
                const size_t e2 = ahead / S, nl = (size_t)a.nel * NP;
                l2_prefetch(a.lam + e2 * NP, NP * sizeof(T), a.lam, a.lam + nl);
                l2_prefetch(a.mu + e2 * NP, NP * sizeof(T), a.mu, a.mu + nl);
                if constexpr (NSLS > 0) l2_prefetch(a.tau + e2 * NP, NP * sizeof(T), a.tau, a.tau + nl);
            }
        }
    }
    for (int x = t; x < 4 * P * P; x += NT) sD[x] = a.tabD[x];

    const int p = t;
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    const size_t nuni = (size_t)a.nuni, nloc = (size_t)a.nloc;
    const size_t li = (size_t)e * NP + p;
    const int ex = e % a.nx, ey = (e / a.nx) % a.ny, ez = e / (a.nx * a.ny);
    const size_t u = unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k);
    const bool act = p < NP && in_range(u, nuni, a.err) && in_range(li, nloc, a.err);
    T vx = 0, vy = 0, vz = 0, lam = 0, mu = 0, tau = 0, cA = 0, cB = 0, cC = 0;
    if (act) {
        const T *vs = a.v + (size_t)s * 3 * nuni;
        vx = vs[u];
        vy = vs[nuni + u];
        vz = vs[2 * nuni + u];
        lam = ld_stream(a.lam + li);
        mu = ld_stream(a.mu + li);
        if constexpr (NSLS > 0) tau = ld_stream(a.tau + li);
        if constexpr (ANISO) {
            cA = ld_stream(a.A + li);
            cB = ld_stream(a.B + li);
            cC = ld_stream(a.C + li);
        }
        sv[p] = vx;
        sv[NP + p] = vy;
        sv[2 * NP + p] = vz;
    }
    __syncthreads();  // velocity slab, derivative tables and the mbarrier's initialisation
    T ev[9];
    if (act) strain_contract<N, T>(sD, sv, sv + NP, sv + 2 * NP, i, j, k, ev);
    // variant_arg bit 0: lane 0 of each warp polls for the whole warp
    const bool landed = (a.variant_arg & 1) ? tma_try_wait_warp(tma_smem(mbar), 0, a.wait_polls)
                                            : tma_try_wait(tma_smem(mbar), 0, a.wait_polls);
    if (act && landed) {
        T sg[6], m[6][MS];
#pragma unroll
        for (int c = 0; c < 6; ++c) sg[c] = st[c * NPS + p];
        if constexpr (NSLS > 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c)
#pragma unroll
                for (int q = 0; q < NSLS; ++q) m[c][q] = st[6 * NPS + (c * NSLS + q) * NPS + p];
        }
        if constexpr (STORE)
            point_update<N, T, NSLS, ANISO, false, true>(a, ev, vx, vy, vz, p, i, j, k, ex, ey, ez, lam, mu, tau, cA,
                                                         cB, cC, sg, m, st + p, st + 6 * NPS + p, NPS, nloc, sf,
                                                         nullptr);
        else
            point_update<N, T, NSLS, ANISO, false, false, KS>(a, ev, vx, vy, vz, p, i, j, k, ex, ey, ez, lam, mu, tau,
                                                              cA, cB, cC, sg, m, a.sig + sb * C::UNIT + p,
                                                              a.mem + sb * C::UNIT + p, NPS, nloc, sf, nullptr,
                                                              KS ? a.sigc + sb * 6 * NPS + p : nullptr);
    }
    // updated state in the stage: visible to the bulk-copy engine after the barrier
    if constexpr (STORE) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const bool ok = __syncthreads_and(landed) != 0;
    if (STORE && ok && t == 0) {
        tma_store(a.sig + sb * C::UNIT, tma_smem(st), C::STAGE_BYTES);
        tma_commit();
    }
    if (ok && act) {
        T fx = 0, fy = 0, fz = 0;
        point_divergence<N, T>(sD + 3 * P * P, sf, i, j, k, fx, fy, fz);
        add_force(a, s, u, fx, fy, fz);
    }
    if (!ok && t == 0) {
        atomicExch(a.err, 1);
        // the copies may still be in flight: one more bounded wait before
        // the block's shared memory is released
        if (issued) tma_try_wait(tma_smem(mbar), 0, a.wait_polls);
    }
    if (STORE && ok && t == 0) tma_wait_read<0>();  // the stores have read the stage before it is released
}

template <int N, typename T, int NSLS, bool ANISO>
int prepare_element_stage() {
    using C = StageCfg<N, T, NSLS>;
    if (C::SMEM <= 48 * 1024) return 0;
    if (C::SMEM > kMaxSmemPerBlock) return 0;
    for (auto *f : {k_element_stage<N, T, NSLS, ANISO, true>, k_element_stage<N, T, NSLS, ANISO, false>,
                    k_element_stage<N, T, NSLS, ANISO, false, true>})
        if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM) != cudaSuccess)
            return -1;
    return 0;
}

// store: 1 bulk store, 0 register stores, -1 the degree's default.
template <int N, typename T, int NSLS, bool ANISO>
int launch_element_stage(const StepArgs<T> &a, int store, void *stream) {
    using C = StageCfg<N, T, NSLS>;
    if (C::SMEM > kMaxSmemPerBlock) return 1;
    const long long blocks = (long long)a.nel * a.S;
    if (a.sigc)
        k_element_stage<N, T, NSLS, ANISO, false, true><<<(unsigned)blocks, C::NT, C::SMEM, (cudaStream_t)stream>>>(a);
    else if (store < 0 ? C::STORE_DEFAULT : store != 0)
        k_element_stage<N, T, NSLS, ANISO, true><<<(unsigned)blocks, C::NT, C::SMEM, (cudaStream_t)stream>>>(a);
    else
        k_element_stage<N, T, NSLS, ANISO, false><<<(unsigned)blocks, C::NT, C::SMEM, (cudaStream_t)stream>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// Resident blocks per SM of the TMA kernel (filled in by prepare, outside capture).
template <int N, typename T, int NSLS, bool ANISO>
struct TmaLaunch {
    static int blocks;
};
template <int N, typename T, int NSLS, bool ANISO>
int TmaLaunch<N, T, NSLS, ANISO>::blocks = 0;

template <int N, typename T, int NSLS, bool ANISO>
int prepare_element_tma() {
    using C = TmaCfg<N, T, NSLS>;
    if (C::SMEM > kMaxSmemPerBlock) return 0;
    cudaError_t e = cudaFuncSetAttribute(k_element_tma<N, T, NSLS, ANISO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)C::SMEM);
    int dev = 0, nb = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_element_tma<N, T, NSLS, ANISO>, C::NT, C::SMEM);
    if (e == cudaSuccess) TmaLaunch<N, T, NSLS, ANISO>::blocks = nb * sms;
    return e == cudaSuccess ? 0 : -1;
}

// Launches the TMA kernel; returns 1 if this configuration has none (the
// caller then falls back to the one-block-per-group kernel).
template <int N, typename T, int NSLS, bool ANISO>
int launch_element_tma(const StepArgs<T> &a, void *stream) {
    using C = TmaCfg<N, T, NSLS>;
    const int resident = TmaLaunch<N, T, NSLS, ANISO>::blocks;
    if (C::SMEM > kMaxSmemPerBlock || resident <= 0) return 1;
    const long long units = (long long)a.nel * a.S;
    const long long blocks = std::min<long long>(units, resident);
    k_element_tma<N, T, NSLS, ANISO><<<(unsigned)blocks, C::NT, C::SMEM, (cudaStream_t)stream>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sesnt
