// Receiver channels and volume-snapshot fields beyond the velocity: the
// rotation strain (the gradient components the reference's rot_v channels
// read after a step), the rotation rate built from it, pressure, and the
// strain of the displacement gradient.
//
// After step it the reference's strain arrays hold the completed gradient of
// the velocity at the start of the step, with exy, exz, eyz symmetrised
// (src/evolution.f90:165-173,206-208), while vx, vy, vz already hold the
// updated velocity; record_rot_v* and get_field('rot_v*')
// (src/config/channel_mod.f90:620-812, src/volume_snapshot.f90:238-246)
// combine exactly those. k_rot_strain recomputes the six components they
// read from the velocity before the node update, for a list of elements (the
// receivers' elements) or for all of them.
#pragma once

namespace sesnt {

// One block per (listed element, simulation).
template <int N, typename T>
__global__ void __launch_bounds__(((N + 1) * (N + 1) * (N + 1) + 31) / 32 * 32)
    k_rot_strain(const StepArgs<T> a, const int *elems, int count, T *out) {
    constexpr int P = N + 1, NP = P * P * P;
    __shared__ T sD[3 * P * P];
    __shared__ T sv[3 * NP];
    const int idx = blockIdx.x, s = blockIdx.y, t = threadIdx.x;
    const int e = elems ? elems[idx] : idx;
    if (!in_range(e, a.nel, a.err)) return;  // whole block
    for (int x = t; x < 3 * P * P; x += blockDim.x) sD[x] = a.tabD[x];
    const int p = t;
    const bool act = p < NP;
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    const int ex = e % a.nx, ey = (e / a.nx) % a.ny, ez = e / (a.nx * a.ny);
    const size_t nuni = (size_t)a.nuni;
    T vx = 0, vy = 0, vz = 0;
    if (act) {
        const size_t u = unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k);
        const T *vs = a.v + (size_t)s * 3 * nuni;
        vx = vs[u];
        vy = vs[nuni + u];
        vz = vs[2 * nuni + u];
        sv[p] = vx;
        sv[NP + p] = vy;
        sv[2 * NP + p] = vz;
    }
    __syncthreads();
    if (!act) return;
    T ev[9], g[9];
    strain_contract<N, T>(sD, sv, sv + NP, sv + 2 * NP, i, j, k, ev);
    complete_gradient<N, T>(a, ev, vx, vy, vz, i, k, ex, ez, g);
    T rs[6];
    rs[kRotEYZ] = (g[kDuYZ] + g[kDuZY]) * T(0.5);
    rs[kRotEZY] = g[kDuZY];
    rs[kRotEZX] = g[kDuZX];
    rs[kRotEXZ] = (g[kDuXZ] + g[kDuZX]) * T(0.5);
    rs[kRotEXY] = (g[kDuXY] + g[kDuYX]) * T(0.5);
    rs[kRotEYX] = g[kDuYX];
#pragma unroll
    for (int c = 0; c < 6; ++c) out[(((size_t)s * 6 + c) * count + idx) * NP + p] = rs[c];
}

// Rotation-rate component c (0 x, 1 y, 2 z) at point (i, ., k) of element
// (ex, ., ez) from its rotation strain rs[6] and updated velocity, in the
// reference's operation order (src/volume_snapshot.f90:238-246).
template <int N, typename T>
__device__ __forceinline__ T rot_value(const StepArgs<T> &a, int c, const T (&rs)[6], T vx, T vy, int i, int k,
                                       int ex, int ez) {
    constexpr int P = N + 1;
    const T r = a.r[ez * P + k], st = a.sin_t[ex * P + i];
    if (c == 0) return -vy / r + rs[kRotEYZ] / (r * st) + rs[kRotEZY];
    if (c == 1) return -rs[kRotEZX] + (vx - rs[kRotEXZ]) / r;
    return (rs[kRotEXY] + vy * a.cot_t[ex * P + i] - rs[kRotEYX] / st) / r;
}

// Element-local derived field of simulation `sim`, one thread per point.
template <int N, typename T>
__global__ void __launch_bounds__(256) k_derived(const StepArgs<T> a, int which, int sim, const T *rot, T *loc) {
    constexpr int P = N + 1, NP = P * P * P;
    const size_t nloc = (size_t)a.nloc;
    const size_t li = (size_t)blockIdx.x * 256 + threadIdx.x;
    if (li >= nloc) return;
    T out = 0;
    if (which == SESNT_FIELD_PRESSURE) {
        // -1.0*(sxx + syy + szz)/3.0 on the stored stresses (xx xy xz yy yz zz)
        const size_t e = li / NP, p = li % NP;
        const T *sg = a.sig + (e * a.S + sim) * (size_t)a.st_unit + p;
        out = (T(-1) * (sg[0] + sg[3 * a.st_cs] + sg[5 * a.st_cs])) / T(3);
    } else if (which >= SESNT_FIELD_EXX && which <= SESNT_FIELD_EZZ) {
        const T *du = a.du + (size_t)sim * 9 * nloc + li;
        switch (which) {
            case SESNT_FIELD_EXX: out = du[kDuXX * nloc]; break;
            case SESNT_FIELD_EXY: out = (du[kDuXY * nloc] + du[kDuYX * nloc]) / T(2); break;
            case SESNT_FIELD_EXZ: out = (du[kDuXZ * nloc] + du[kDuZX * nloc]) / T(2); break;
            case SESNT_FIELD_EYY: out = du[kDuYY * nloc]; break;
            case SESNT_FIELD_EYZ: out = (du[kDuYZ * nloc] + du[kDuZY * nloc]) / T(2); break;
            default: out = du[kDuZZ * nloc]; break;
        }
    } else {
        const int e = (int)(li / NP), p = (int)(li % NP);
        const int i = p % P, j = (p / P) % P, k = p / (P * P);
        const int ex = e % a.nx, ey = (e / a.nx) % a.ny, ez = e / (a.nx * a.ny);
        const size_t nuni = (size_t)a.nuni;
        const size_t u = unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k);
        const T *vs = a.v + (size_t)sim * 3 * nuni;
        T rs[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) rs[c] = rot[((size_t)sim * 6 + c) * nloc + li];
        out = rot_value<N, T>(a, which - SESNT_FIELD_ROT_VX, rs, vs[u], vs[nuni + u], i, k, ex, ez);
    }
    loc[li] = out;
}

// Receiver channels beyond vx, vy, vz for receiver r of simulation s at step
// it, one warp (called from k_receivers, all lanes): the rotation rates from
// the rotation strain of the receiver's element, and the recorded source
// fields record_m** / record_f* (src/config/channel_mod.f90:859-1095), i.e.
// the slab the sources of this step's add(it) left in the receiver's element.
template <int N, typename T>
__device__ __forceinline__ void record_extra(const StepArgs<T> &a, int r, int s, int it, int lane, int ex, int ey,
                                             int ez, const T *vm) {
    constexpr int P = N + 1, NP = P * P * P;
    const unsigned xm = a.rec_xmask[r];
    if (!xm) return;
    int slot = a.rec_xslot[r];
    if (!in_range(slot + __popc(xm) - 1, a.nxtr, a.err)) return;  // whole warp
    T *xo = a.xseis + (size_t)s * a.nxtr * a.nt + (it - 1);
    const size_t nuni = (size_t)a.nuni;
    auto reduce = [](T x) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        return x;
    };
    if (xm & (SESNT_CH_ROT_VX | SESNT_CH_ROT_VY | SESNT_CH_ROT_VZ)) {
        const int rr = a.rec_rot[r];
        if (!in_range(rr, a.nrot, a.err)) return;
        const T *vs = a.v + (size_t)s * 3 * nuni;
        for (int c = 0; c < 3; ++c) {
            if (!(xm & (SESNT_CH_ROT_VX << c))) continue;
            T acc = 0;
            for (int p = lane; p < NP; p += 32) {
                const int i = p % P, j = (p / P) % P, k = p / (P * P);
                const size_t u = unique_index<N>(a.NXU, a.NYU, ex, ey, ez, i, j, k);
                T rs[6];
#pragma unroll
                for (int q = 0; q < 6; ++q) rs[q] = a.rot_rec[(((size_t)s * 6 + q) * a.nrot + rr) * NP + p];
                acc += vm[p] * rot_value<N, T>(a, c, rs, vs[u], vs[nuni + u], i, k, ex, ez);
            }
            acc = reduce(acc);
            if (lane == 0) xo[(size_t)slot * a.nt] = acc;
            ++slot;
        }
    }
    const int ri = a.rec_src ? a.rec_src[(size_t)s * a.nrec + r] : -1;
    for (int c = 0; c < 9; ++c) {
        if (!(xm & (SESNT_CH_MXX << c))) continue;
        T acc = 0;
        if (ri >= 0 && in_range(ri, a.nsrc, a.err)) {
            const SrcRec rec = a.src[ri];
            if (rec.vm[c] >= 0 && in_range(rec.vm[c], a.n_src_vm, a.err) && in_range(rec.data[c], a.n_src_data, a.err)) {
                const T d = a.src_data[(size_t)rec.data[c] * a.nt + (it - 1)];
                const T *svm = a.src_vm + (size_t)rec.vm[c] * NP;
                for (int p = lane; p < NP; p += 32) {
                    const int i = p % P, j = (p / P) % P, k = p / (P * P);
                    T val;
                    if (c < 6) {
                        const T rr = a.r[ez * P + k];
                        const T rr2 = rr * (rr * a.sin_t[ex * P + i]);
                        const T W = a.w[i] * a.w[j] * a.w[k];
                        val = (-d * svm[p]) / (a.jac * W * rr2);
                    } else {
                        val = -d * svm[p];
                    }
                    acc += vm[p] * val;
                }
            }
        }
        acc = reduce(acc);
        if (lane == 0) xo[(size_t)slot * a.nt] = acc;
        ++slot;
    }
}

template <int N, typename T>
int launch_rot_strain(const StepArgs<T> &a, const int *elems, int count, T *out, void *stream) {
    if (count <= 0) return 0;
    constexpr int NP = (N + 1) * (N + 1) * (N + 1);
    dim3 grid((unsigned)count, (unsigned)a.S);
    k_rot_strain<N, T><<<grid, (NP + 31) / 32 * 32, 0, (cudaStream_t)stream>>>(a, elems, count, out);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int N, typename T>
int launch_derived(const StepArgs<T> &a, int which, int sim, const T *rot, T *loc, void *stream) {
    k_derived<N, T><<<(unsigned)((a.nloc + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a, which, sim, rot, loc);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sesnt
