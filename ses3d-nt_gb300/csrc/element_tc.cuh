// Tensor-core variant of the element kernel (FP32 wavefields): the nine
// velocity-gradient line contractions and the nine weak-divergence line
// contractions of an element run as tcgen05.mma products in split precision
// with FP32 accumulation, beside the CUDA-core kernel.
//
// A contraction along one GLL direction is out[line, n] = sum_q A[line, q]
// B[q, n] over the element's lines (the two other GLL indices) and the three
// components: rows = 3 directions x P^2 lines x 3 components = 9 P^2,
// K = q (P <= 8, padded to 8 for TF32 and 16 for BF16), N = n padded to 16.
// Rows are packed into M = 128 tiles; A and B sit in shared memory in the
// no-swizzle K-major canonical layout (8-row x 16-byte core matrices, K
// chunks 128 B apart, 8-row groups 256 B apart); D accumulates in TMEM.
//   TF32x3:  a = a_hi + a_lo (tf32 parts), D = a_lo b_hi + a_hi b_lo + a_hi b_hi
//   BF16x3:  the same with bf16 parts
// B for the gradient is l_q'(xi_n) (scaled by 2/d_elm afterwards); B for the
// divergence is l_n'(xi_q).
#pragma once

#include <cuda_bf16.h>

namespace sesnt {

template <int N, int PREC>  // PREC 1: TF32x3, 2: BF16x3
struct TcCfg {
    static constexpr int P = N + 1, NP = P * P * P;
    static constexpr int ROWS = 9 * P * P;
    static constexpr int TILES = (ROWS + 127) / 128;
    static constexpr int NT = ((NP + 127) / 128) * 128;  // whole warp quadrants
    static constexpr int NW = NT / 32;
    static constexpr int EB = PREC == 1 ? 4 : 2;  // bytes per operand element
    static constexpr int TILE_BYTES = 4096;       // 128 rows x 32 bytes
    static constexpr int A_BYTES = TILES * TILE_BYTES;
    static constexpr int B_BYTES = 512;           // 16 rows x 32 bytes
    static constexpr int COLS_PER_PASS = TILES * 16;
    static constexpr int TMEM_COLS = COLS_PER_PASS * 2 <= 32 ? 32
                                     : (COLS_PER_PASS * 2 <= 64 ? 64 : (COLS_PER_PASS * 2 <= 128 ? 128 : 256));
    // shared memory: A hi/lo, B hi/lo (gradient, divergence), 16 bytes for
    // the mbarrier and TMEM address, the derivative tables (padded to 16 B)
    // and a 9 x NP float exchange slab
    static constexpr size_t TAB_BYTES = ((4 * P * P * 4 + 15) / 16) * 16;
    static constexpr size_t SMEM = 2 * A_BYTES + 4 * B_BYTES + 16 + TAB_BYTES + 9 * NP * 4;
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory descriptor: no swizzle, K-major, version 1.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// tcgen05 instruction descriptor: D f32, A/B of `ab` (1 bf16, 2 tf32),
// K-major A and B, M = 128, N = 16.
__device__ __forceinline__ uint32_t tc_idesc(uint32_t ab) {
    return (1u << 4) | (ab << 7) | (ab << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
}

// Byte offset of (row, q) in a stack of 128-row K-major tiles.
template <int EB>
__device__ __forceinline__ int tc_off(int row, int q) {
    const int r = row & 127;
    return (row >> 7) * 4096 + (r & 7) * 16 + (r >> 3) * 256 + ((q * EB) >> 4) * 128 + ((q * EB) & 15);
}

template <int PREC>
__device__ __forceinline__ void tc_split_store(unsigned char *hi, unsigned char *lo, int off, float x) {
    if constexpr (PREC == 1) {
        uint32_t h;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
        const float hf = __uint_as_float(h);
        uint32_t l;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(x - hf));
        *reinterpret_cast<uint32_t *>(hi + off) = h;
        *reinterpret_cast<uint32_t *>(lo + off) = l;
    } else {
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
        *reinterpret_cast<__nv_bfloat16 *>(hi + off) = h;
        *reinterpret_cast<__nv_bfloat16 *>(lo + off) = l;
    }
}

// Bounded wait for the mbarrier phase `parity` (at most `polls` polls);
// false when it ran out.
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity, int polls) {
    uint32_t done = 0;
    for (int it = 0; it < polls && !done; ++it)
        asm volatile(
            "{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p;}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
    return done != 0;
}

// Issue the three split products for every tile, accumulating into TMEM
// columns col0 + 16*tile, then commit to the mbarrier. One thread.
template <int PREC, int TILES>
__device__ __forceinline__ void tc_issue(uint32_t tmem, uint32_t col0, const unsigned char *a_hi,
                                         const unsigned char *a_lo, const unsigned char *b_hi,
                                         const unsigned char *b_lo, uint32_t mbar) {
    const uint32_t id = tc_idesc(PREC == 1 ? 2u : 1u);
    const uint64_t bh = tc_sdesc(smem_addr(b_hi), 128, 256), bl = tc_sdesc(smem_addr(b_lo), 128, 256);
#pragma unroll
    for (int t = 0; t < TILES; ++t) {
        const uint64_t ah = tc_sdesc(smem_addr(a_hi + t * 4096), 128, 256);
        const uint64_t al = tc_sdesc(smem_addr(a_lo + t * 4096), 128, 256);
        const uint32_t d = tmem + col0 + 16 * t;
        const uint64_t as_[3] = {al, ah, ah}, bs_[3] = {bh, bl, bh};  // small products first
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const uint32_t acc = r > 0;
            if constexpr (PREC == 1)
                asm volatile(
                    "{.reg .pred p; setp.ne.u32 p, %4, 0; tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;}" ::"r"(d),
                    "l"(as_[r]), "l"(bs_[r]), "r"(id), "r"(acc));
            else
                asm volatile(
                    "{.reg .pred p; setp.ne.u32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;}" ::"r"(d),
                    "l"(as_[r]), "l"(bs_[r]), "r"(id), "r"(acc));
        }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// Row of a contraction tile: direction d (0 x, 1 y, 2 z), line (the two other
// GLL indices), component c. The point of output n of that row.
template <int P>
__device__ __forceinline__ int tc_point(int d, int line, int n) {
    if (d == 0) return n + P * line;                          // line = j + P*k
    if (d == 1) return (line % P) + P * (n + P * (line / P));  // line = i + P*k
    return line + P * P * n;                                  // line = i + P*j
}

// Read this warp's quadrant of every tile it owns (tcgen05.ld 32x32b.x16)
// and scatter the P outputs of each row to slab[(d*3 + c)*NP + point],
// scaled by scale[d].
template <int N, int PREC>
__device__ __forceinline__ void tc_read_rows(uint32_t tmem, uint32_t col0, float *slab, const float scale[3]) {
    using C = TcCfg<N, PREC>;
    constexpr int P = C::P, NP = C::NP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, quad = warp & 3;
    for (int t = warp >> 2; t < C::TILES; t += C::NW / 4) {
        uint32_t v[16];
        const uint32_t addr = tmem + ((uint32_t)(quad * 32) << 16) + col0 + 16 * t;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(addr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        const int row = t * 128 + quad * 32 + lane;
        if (row < C::ROWS) {
            const int d = row / (3 * P * P), rest = row - d * 3 * P * P, line = rest / 3, c = rest - line * 3;
#pragma unroll
            for (int n = 0; n < P; ++n) slab[(d * 3 + c) * NP + tc_point<P>(d, line, n)] = __uint_as_float(v[n]) * scale[d];
        }
    }
}

// One block per (element, simulation); thread p owns point p (p < NP).
template <int N, int NSLS, bool ANISO, int PREC>
__global__ void __launch_bounds__(TcCfg<N, PREC>::NT) k_element_tc(const StepArgs<float> a) {
    using C = TcCfg<N, PREC>;
    using T = float;
    constexpr int P = C::P, NP = C::NP, MS = NSLS > 0 ? NSLS : 1, EB = C::EB;
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char *a_hi = tc_smem, *a_lo = a_hi + C::A_BYTES;
    unsigned char *bg_hi = a_lo + C::A_BYTES, *bg_lo = bg_hi + C::B_BYTES;
    unsigned char *bd_hi = bg_lo + C::B_BYTES, *bd_lo = bd_hi + C::B_BYTES;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(bd_lo + C::B_BYTES);  // 512-byte aligned
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 1);
    float *sD = reinterpret_cast<float *>(bd_lo + C::B_BYTES + 16);      // [4][P*P]
    float *slab = reinterpret_cast<float *>(bd_lo + C::B_BYTES + 16 + C::TAB_BYTES);  // [9][NP]

    const int t = threadIdx.x, warp = t >> 5;
    const int S = a.S;
    const int s = blockIdx.x % S;
    const int e = blockIdx.x / S;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "n"(C::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    for (int x = t; x < 4 * P * P; x += C::NT) sD[x] = a.tabD[x];
    // zero the operands once (K and N padding must be 0, never NaN)
    for (int x = t; x < (2 * C::A_BYTES + 4 * C::B_BYTES) / 16; x += C::NT)
        reinterpret_cast<uint4 *>(tc_smem)[x] = make_uint4(0, 0, 0, 0);
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // B operands: row n of B^T holds B[q][n] along q
    const float *dl = a.tabD + 3 * P * P;  // dl[i*P+q] = l_i'(xi_q)
    if (t < 16) {
        for (int q = 0; q < P && t < P; ++q) {
            tc_split_store<PREC>(bg_hi, bg_lo, tc_off<EB>(t, q), dl[q * P + t]);  // gradient: l_q'(xi_n)
            tc_split_store<PREC>(bd_hi, bd_lo, tc_off<EB>(t, q), dl[t * P + q]);  // divergence: l_n'(xi_q)
        }
    }

    const int p = t;
    const bool act = p < NP;
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    const int ex = e % a.nx, ey = (e / a.nx) % a.ny, ez = e / (a.nx * a.ny);
    const size_t nuni = (size_t)a.nuni, nloc = (size_t)a.nloc;
    const size_t li = (size_t)e * NP + p;
    size_t u = 0;
    T vx = 0, vy = 0, vz = 0, lam = 0, mu = 0, tau = 0, cA = 0, cB = 0, cC = 0;
    T sg[6] = {0, 0, 0, 0, 0, 0}, m[6][MS];
    constexpr int NPS = StateLayout<NP, NSLS>::CS;  // element-blocked units (StateLayout)
    T *sig = a.sig + ((size_t)e * S + s) * StateLayout<NP, NSLS>::UNIT + p;
    T *mem = a.mem + ((size_t)e * S + s) * StateLayout<NP, NSLS>::UNIT + p;
    if (act && in_range(unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k), nuni, a.err) &&
        in_range(li, nloc, a.err)) {
        u = unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k);
        const T *vs = a.v + (size_t)s * 3 * nuni;
        vx = vs[u];
        vy = vs[nuni + u];
        vz = vs[2 * nuni + u];
        lam = ld_stream(a.lam + li);
        mu = ld_stream(a.mu + li);
        if constexpr (ANISO) {
            cA = ld_stream(a.A + li);
            cB = ld_stream(a.B + li);
            cC = ld_stream(a.C + li);
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) sg[c] = ld_stream(sig + c * NPS);
        if constexpr (NSLS > 0) {
            tau = ld_stream(a.tau + li);
#pragma unroll
            for (int c = 0; c < 6; ++c)
#pragma unroll
                for (int q = 0; q < NSLS; ++q) m[c][q] = ld_stream(mem + (size_t)(c * NSLS + q) * NPS);
        }
        // velocity into the gradient operand: x rows (j,k), y rows (i,k), z rows (i,j)
        const T vv[3] = {vx, vy, vz};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            tc_split_store<PREC>(a_hi, a_lo, tc_off<EB>(0 * 3 * P * P + (j + P * k) * 3 + c, i), vv[c]);
            tc_split_store<PREC>(a_hi, a_lo, tc_off<EB>(1 * 3 * P * P + (i + P * k) * 3 + c, j), vv[c]);
            tc_split_store<PREC>(a_hi, a_lo, tc_off<EB>(2 * 3 * P * P + (i + P * j) * 3 + c, k), vv[c]);
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    if (t == 0 && !a.drop_completion) tc_issue<PREC, C::TILES>(tmem, 0, a_hi, a_lo, bg_hi, bg_lo, smem_addr(mbar));
    // block-uniform outcome: tcgen05.ld below is warp-collective
    const bool ok1 = __syncthreads_and(tc_wait(smem_addr(mbar), 0, a.wait_polls)) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const float gscale[3] = {a.two_over_d[0], a.two_over_d[1], a.two_over_d[2]};
    if (ok1) tc_read_rows<N, PREC>(tmem, 0, slab, gscale);
    __syncthreads();
    if (act && ok1) {  // without the gradient the point keeps its state
        T ev[9];
        // slab[(d*3 + c)*NP + p] = d-derivative of component c: the layout of strain_contract
#pragma unroll
        for (int q = 0; q < 9; ++q) ev[q] = slab[q * NP + p];
        point_update<N, T, NSLS, ANISO>(a, ev, vx, vy, vz, p, i, j, k, ex, ey, ez, lam, mu, tau, cA, cB, cC, sg, m,
                                        sig, mem, NPS, nloc, slab, nullptr);
        // fluxes slab[(c*3 + d)*NP + p] (force component c, direction d) into the divergence operand
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            tc_split_store<PREC>(a_hi, a_lo, tc_off<EB>(0 * 3 * P * P + (j + P * k) * 3 + c, i), slab[(c * 3 + 0) * NP + p]);
            tc_split_store<PREC>(a_hi, a_lo, tc_off<EB>(1 * 3 * P * P + (i + P * k) * 3 + c, j), slab[(c * 3 + 1) * NP + p]);
            tc_split_store<PREC>(a_hi, a_lo, tc_off<EB>(2 * 3 * P * P + (i + P * j) * 3 + c, k), slab[(c * 3 + 2) * NP + p]);
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (t == 0 && ok1) tc_issue<PREC, C::TILES>(tmem, C::COLS_PER_PASS, a_hi, a_lo, bd_hi, bd_lo, smem_addr(mbar));
    const bool ok = __syncthreads_and(ok1 && tc_wait(smem_addr(mbar), 1, a.wait_polls)) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const float one[3] = {1.0f, 1.0f, 1.0f};
    if (ok) tc_read_rows<N, PREC>(tmem, C::COLS_PER_PASS, slab, one);
    __syncthreads();
    if (!ok) {
        // record the failure; give the products still in flight one more
        // bounded wait before the accumulator columns are freed
        if (t == 0) atomicExch(a.err, 1);
        tc_wait(smem_addr(mbar), ok1 ? 1u : 0u, a.wait_polls);
    }
    if (act && ok) {
        // slab[(d*3 + c)*NP + p]: direction-d part of force component c
        const T fx = slab[0 * NP + p] + slab[3 * NP + p] + slab[6 * NP + p];
        const T fy = slab[1 * NP + p] + slab[4 * NP + p] + slab[7 * NP + p];
        const T fz = slab[2 * NP + p] + slab[5 * NP + p] + slab[8 * NP + p];
        add_force(a, s, u, fx, fy, fz);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(C::TMEM_COLS));
}

template <int N, int NSLS, bool ANISO, int PREC>
int launch_element_tc_v(const StepArgs<float> &a, void *stream) {
    using C = TcCfg<N, PREC>;
    const long long blocks = (long long)a.nel * a.S;
    k_element_tc<N, NSLS, ANISO, PREC><<<(unsigned)blocks, C::NT, C::SMEM, (cudaStream_t)stream>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int N, int PREC>
int prepare_element_tc() {
    using C = TcCfg<N, PREC>;
    if (C::SMEM <= 48 * 1024) return 0;
    cudaError_t e = cudaFuncSetAttribute(k_element_tc<N, 0, false, PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_element_tc<N, 0, true, PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_element_tc<N, kNsls, false, PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_element_tc<N, kNsls, true, PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    return e == cudaSuccess ? 0 : -1;
}

template <int N>
int launch_element_tc(const StepArgs<float> &a, bool sls, bool aniso, void *stream) {
    if (a.contraction == 1) {
        if (sls) return aniso ? launch_element_tc_v<N, kNsls, true, 1>(a, stream) : launch_element_tc_v<N, kNsls, false, 1>(a, stream);
        return aniso ? launch_element_tc_v<N, 0, true, 1>(a, stream) : launch_element_tc_v<N, 0, false, 1>(a, stream);
    }
    if (sls) return aniso ? launch_element_tc_v<N, kNsls, true, 2>(a, stream) : launch_element_tc_v<N, kNsls, false, 2>(a, stream);
    return aniso ? launch_element_tc_v<N, 0, true, 2>(a, stream) : launch_element_tc_v<N, 0, false, 2>(a, stream);
}

}  // namespace sesnt
