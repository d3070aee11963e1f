// Oracle for the Ses3d-NT spectral-element time step: a CPU restatement of the
// reference Fortran, kept in the reference's own rank-6 layout
// f(0:nx-1, 0:ny-1, 0:nz-1, 0:N, 0:N, 0:N) (Fortran order, element x fastest).
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU library: it
// is compiled into oracle/_build/liboracle.so and loaded only by tests/,
// __graft_entry__.smoke() and the CPU-baseline leg of bench.py. The product
// library never links, loads or calls it.
//
// Every routine names the reference file:line it restates. Floating-point
// expressions keep the reference's evaluation order (Fortran evaluates left
// to right; `a**2` is a*a), and the file is compiled with
// -ffp-contract=off so no multiply-add is fused that the reference would
// round twice.
//
// Pinned: the GLL tables, coordinates, Lagrange interpolation and assembly
// map, against the reference's own unit programs under src/examples/
// (gll_test, coordinates_test, interpolation_test) and its tabulated
// constants, in tests/test_oracle_pins.py.
// Parity unpinned for the time step itself: the reference ships no solver
// tests, seismograms or golden wavefields, and it is Fortran + MPI with no
// compiler available, so it cannot be run to produce them.
//
// The visco-elastic (standard linear solid) branch is commented out in the
// reference (src/evolution.f90:216-284,415-442). It is restated here from
// those comments with one fix: the off-diagonal memory sums at :266-268 add
// Mxx/Myy/Mzz where Mxy/Mxz/Myz are meant (compare the loop at :258-264).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// GLL knots and weights: src/gll_mod.f90:61-165 (closed forms for lpd 1..6,
// 16-digit literals for lpd 7), evaluated in the working precision T the
// way a Fortran compiler folds the constant expressions.
// ---------------------------------------------------------------------------
template <class T>
std::vector<T> gll_knots(int lpd) {
    // size lpd+1 (an array of size 1 for lpd = 0, empty below), as the
    // explicit-shape result knots(lpd+1) of get_knots (:178-201)
    std::vector<T> k(lpd >= 0 ? lpd + 1 : 0, T(0));
    const T one = 1, two = 2;
    switch (lpd) {
        case 1: k = {-one, one}; break;
        case 2: k = {-one, T(0), one}; break;
        case 3: { T a = std::sqrt(one / T(5)); k = {-one, -a, a, one}; } break;
        case 4: { T a = std::sqrt(T(3) / T(7)); k = {-one, -a, T(0), a, one}; } break;
        case 5: {
            T s7 = std::sqrt(T(7)), s21 = std::sqrt(T(21));
            T a = std::sqrt(two * s7 + T(7)) / s21;
            T b = std::sqrt(T(7) - two * s7) / s21;
            k = {-one, -a, -b, b, a, one};
        } break;
        case 6: {
            T s15 = std::sqrt(T(15)), s33 = std::sqrt(T(33));
            T a = std::sqrt(two * s15 + T(15)) / s33;
            T b = std::sqrt(T(15) - two * s15) / s33;
            k = {-one, -a, -b, T(0), b, a, one};
        } break;
        case 7:
            k = {-one, T(-0.8717401485096066), T(-0.5917001814331423), T(-0.2092992179024789),
                 T(0.2092992179024789), T(0.5917001814331423), T(0.8717401485096066), one};
            break;
        default: break;  // lpd > 7: zeros (src/gll_mod.f90:197-199)
    }
    return k;
}

template <class T>
std::vector<T> gll_weights(int lpd) {
    std::vector<T> w(lpd >= 0 ? lpd + 1 : 0, T(0));
    const T one = 1;
    switch (lpd) {
        case 1: w = {T(0.5), T(0.5)}; break;
        case 2: w = {one / T(3), T(4) / T(3), one / T(3)}; break;
        case 3: w = {one / T(6), T(5) / T(6), T(5) / T(6), one / T(6)}; break;
        case 4: w = {one / T(10), T(49) / T(90), T(32) / T(45), T(49) / T(90), one / T(10)}; break;
        case 5: {
            T s7 = std::sqrt(T(7));
            T a = T(63) / (T(10) * s7 + T(140));
            T b = -T(63) / (T(10) * s7 - T(140));
            w = {one / T(15), a, b, b, a, one / T(15)};
        } break;
        case 6: {
            T s15 = std::sqrt(T(15));
            T a = T(14641) / (T(2450) * s15 + T(43400));
            T b = -T(14641) / (T(2450) * s15 - T(43400));
            w = {one / T(21), a, b, T(256) / T(525), b, a, one / T(21)};
        } break;
        case 7:
            w = {T(0.0357142857142857), T(0.2107042271435061), T(0.3411226924835044),
                 T(0.4124587946587038), T(0.4124587946587038), T(0.3411226924835044),
                 T(0.2107042271435061), T(0.0357142857142857)};
            break;
        default: break;
    }
    return w;
}

// get_dlgll: src/gll_mod.f90:251-275. Derivative of Lagrange polynomial i at
// collocation point j.
template <class T>
T get_dlgll(int n, int i, int j) {
    std::vector<T> knots = gll_knots<T>(n);
    T xi = knots[i], xj = knots[j];
    std::vector<T> xk;
    for (T v : knots)
        if (v != xi) xk.push_back(v);
    T y;
    if (i == j) {
        y = 0;
        for (T v : xk) y = y + T(1) / (xi - v);
    } else {
        T num = 1, den = 1;
        for (T v : xk)
            if (v != xj) num = num * (xj - v);
        for (T v : xk) den = den * (xi - v);
        y = num / den;
    }
    return y;
}

// coordinates_1d: src/coordinates_mod.f90:114-141. Returns coords[e*(lpd+1)+j].
template <class T>
std::vector<T> coordinates_1d(int elms, int lpd, T mn, T mx) {
    std::vector<T> knots = gll_knots<T>(lpd);
    for (auto &k : knots) k = T(0.5) * (T(1) + k);
    T delta = (mx - mn) / T(elms);
    std::vector<T> c((size_t)elms * (lpd + 1));
    for (int i = 0; i < elms; ++i)
        for (int j = 0; j <= lpd; ++j) c[(size_t)i * (lpd + 1) + j] = mn + (T(i) + knots[j]) * delta;
    c[(size_t)(elms - 1) * (lpd + 1) + lpd] = mx;  // "XXX hack" :139
    return c;
}

template <class T>
T pi_() { return T(2) * std::acos(T(0)); }  // src/parameters.F90:67

template <class T>
T deg2rad(T d) { return d * pi_<T>() / T(180); }  // src/misc/coordinate_utilities_mod.f90:79-82

// Domain extents on one rank: src/config/model.f90:90-237 with px=py=pz=1 and
// mpi_*_coord=0. Note x_loc_max = x_glb_min + dx_glb, which can differ from
// x_glb_max in the last bit; the reference uses each where it does.
template <class T>
struct Extents {
    T x_glb_min, x_glb_max, y_glb_min, y_glb_max, z_glb_min, z_glb_max;
    T dx_elm, dy_elm, dz_elm;
    T x_loc_min, x_loc_max, y_loc_min, y_loc_max, z_loc_min, z_loc_max;
};

template <class T>
Extents<T> make_extents(int nx, int ny, int nz, T lat_min, T lat_max, T lon_min, T lon_max, T rad_min,
                        T rad_max) {
    Extents<T> e;
    e.x_glb_min = deg2rad<T>(T(90) - lat_max);
    e.x_glb_max = deg2rad<T>(T(90) - lat_min);
    e.y_glb_min = deg2rad<T>(lon_min);
    e.y_glb_max = deg2rad<T>(lon_max);
    e.z_glb_min = rad_min;
    e.z_glb_max = rad_max;
    T dx_glb = e.x_glb_max - e.x_glb_min, dy_glb = e.y_glb_max - e.y_glb_min, dz_glb = e.z_glb_max - e.z_glb_min;
    T dx_loc = dx_glb / T(1), dy_loc = dy_glb / T(1), dz_loc = dz_glb / T(1);
    e.dx_elm = dx_glb / T(nx);
    e.dy_elm = dy_glb / T(ny);
    e.dz_elm = dz_glb / T(nz);
    e.x_loc_min = e.x_glb_min + T(0) * dx_loc;
    e.x_loc_max = e.x_glb_min + T(1) * dx_loc;
    e.y_loc_min = e.y_glb_min + T(0) * dy_loc;
    e.y_loc_max = e.y_glb_min + T(1) * dy_loc;
    e.z_loc_min = e.z_glb_min + T(0) * dz_loc;
    e.z_loc_max = e.z_glb_min + T(1) * dz_loc;
    return e;
}

// Lagrange interpolation: src/interpolation_mod.f90:83-171.
template <class T>
std::vector<T> lagrange(T x, const std::vector<T> &knots) {
    size_t n = knots.size();
    std::vector<T> l(n, T(1));
    if (n <= 1) return l;
    std::vector<T> w(n);
    for (size_t j = 0; j < n; ++j) {  // calc_weights :83-91
        T p1 = 1, p2 = 1;
        for (size_t i = 0; i < j; ++i) p1 = p1 * (knots[j] - knots[i]);
        for (size_t i = j + 1; i < n; ++i) p2 = p2 * (knots[j] - knots[i]);
        w[j] = T(1) / (p1 * p2);
    }
    bool all_diff = true;
    for (size_t j = 0; j < n; ++j)
        if (!(x != knots[j])) all_diff = false;
    if (all_diff) {
        T prod = 1;
        for (size_t j = 0; j < n; ++j) prod = prod * (x - knots[j]);
        for (size_t j = 0; j < n; ++j) l[j] = prod / (x - knots[j]) * w[j];
    } else {
        for (size_t j = 0; j < n; ++j) l[j] = (x != knots[j]) ? T(0) : T(1);
    }
    return l;
}

template <class T>
void par_range(size_t n, const auto &fn) {
#ifdef _OPENMP
#pragma omp parallel
    {
        int nt = omp_get_num_threads(), id = omp_get_thread_num();
        size_t chunk = (n + nt - 1) / nt, a = std::min(n, chunk * id), b = std::min(n, a + chunk);
        if (a < b) fn(a, b);
    }
#else
    fn(size_t(0), n);
#endif
}

// communicate_local_boundaries: src/communicate_fields.F90:48-79.
// Sequential theta, phi, r passes over shared faces.
template <class T>
void assemble_local(T *f, int nx, int ny, int nz, int N) {
    const int P = N + 1;
    const size_t nel = (size_t)nx * ny * nz;
    auto I = [&](int ex, int ey, int ez, int i, int j, int k) -> size_t {
        return (size_t)ex + (size_t)nx * (ey + (size_t)ny * ez) + nel * (i + (size_t)P * (j + (size_t)P * k));
    };
    for (int ex = 1; ex < nx; ++ex)
        for (int k = 0; k < P; ++k)
            for (int j = 0; j < P; ++j)
                for (int ez = 0; ez < nz; ++ez)
                    for (int ey = 0; ey < ny; ++ey) {
                        size_t a = I(ex, ey, ez, 0, j, k), b = I(ex - 1, ey, ez, N, j, k);
                        f[a] = f[a] + f[b];
                        f[b] = f[a];
                    }
    for (int ey = 1; ey < ny; ++ey)
        for (int k = 0; k < P; ++k)
            for (int i = 0; i < P; ++i)
                for (int ez = 0; ez < nz; ++ez)
                    for (int ex = 0; ex < nx; ++ex) {
                        size_t a = I(ex, ey, ez, i, 0, k), b = I(ex, ey - 1, ez, i, N, k);
                        f[a] = f[a] + f[b];
                        f[b] = f[a];
                    }
    for (int ez = 1; ez < nz; ++ez)
        for (int j = 0; j < P; ++j)
            for (int i = 0; i < P; ++i)
                for (int ey = 0; ey < ny; ++ey)
                    for (int ex = 0; ex < nx; ++ex) {
                        size_t a = I(ex, ey, ez, i, j, 0), b = I(ex, ey, ez - 1, i, j, N);
                        f[a] = f[a] + f[b];
                        f[b] = f[a];
                    }
}

// Source-time functions: src/misc/source_signature_mod.f90:50-147, sampled at
// t = (it-1)*dt as in src/config/source.f90:583-586.
template <class T>
void source_signature(int kind, T onset, T width, T dt, int nt, T *out) {
    const T pi = pi_<T>();
    for (int i = 0; i < nt; ++i) {
        T t = T(i) * dt, s = 0;
        switch (kind) {
            case 0:  // DELTA
                s = (t == onset) ? T(1) : T(0);
                break;
            case 1: {  // RICKER
                T q = pi / width;
                T a2 = -(q * q);
                T d = t - onset;
                s = T(2) * (T(0.5) + a2 * (d * d)) * std::exp(a2 * (d * d));
            } break;
            case 2: {  // GAUSS
                T d = (t - onset) / width;
                s = std::exp(-(d * d));
            } break;
            case 3:  // SIN**3
                if (onset < t && t < onset + width) {
                    T v = std::sin(pi * (t - onset) / width);
                    s = v * v * v;
                } else {
                    s = 0;
                }
                break;
            case 4:  // BRUNE
                if (t >= onset)
                    s = (t - onset) / (width * width) * std::exp(-(t - onset) / width);
                else
                    s = 0;
                break;
            default: s = 0;
        }
        out[i] = s;
    }
}

// ---------------------------------------------------------------------------
// The simulation state and one time step.
// ---------------------------------------------------------------------------
template <class T>
struct Sim {
    using real_t = T;
    int nx, ny, nz, N, P, NP, nt, pml;
    size_t nel, nloc;
    T dt, alpha, jac;
    Extents<T> ext;
    std::vector<T> dl;  // dl[i*P+j] = get_dlgll(N,i,j)
    std::vector<T> x1, y1, z1;  // 1-D coordinates [e*P+n]
    std::vector<T> r, sin_t, cot_t, r_sin, rr_sin, W, taper;
    std::vector<T> lambda, mu, rhoinv, A, B, C, qq, two_mu, kappa, tau, mu_tau, MM, rho;
    bool visco = false;
    static constexpr int nrdiss = 3;
    T tau_p[3] = {T(1000.00), T(70.00), T(5.25)};  // src/geometric_paras.f90:41-42
    // state
    std::vector<T> vx, vy, vz, sx, sy, sz;
    std::vector<T> sxx, sxy, sxz, syy, syz, szz;  // the reference's *_pml stresses
    std::vector<T> exx, eyy, ezz, exy, eyx, exz, ezx, ezy, eyz;
    std::vector<T> M[6][3];  // memory variables xx,yy,zz,xy,xz,yz per relaxation mechanism
    std::vector<T> src[9];   // src_xx,xy,xz,yy,yz,zz, src_x,y,z
    std::vector<T> L, txx, txy, txz, tyy, tyz, tzz;  // step temporaries (automatic arrays at :109-119)
    struct Channel { int comp; std::vector<T> data; };
    struct Source { int ex, ey, ez; std::vector<T> vm; std::vector<Channel> ch; };
    // displacement gradient (src/elastic_vars.F90, integrated at
    // src/evolution.f90:179-187), kept when keep_du is set
    bool keep_du = false;
    std::vector<T> dxux, dyuy, dzuz, dxuy, dyux, dxuz, dzux, dyuz, dzuy;
    // channel bit b (b = 0..15, as the receiver channel mask) -> data; vx, vy,
    // vz always recorded in data[0..2]
    struct Receiver { int ex, ey, ez; unsigned mask; std::vector<T> vm; std::vector<T> data[16]; };
    std::vector<Source> sources;
    std::vector<Receiver> receivers;
    int it = 0;

    size_t I(size_t e, int i, int j, int k) const { return e + nel * (i + (size_t)P * (j + (size_t)P * k)); }
    size_t E(int ex, int ey, int ez) const { return (size_t)ex + (size_t)nx * (ey + (size_t)ny * ez); }

    // init_geometric_parameters: src/geometric_paras.f90:108-325 (one rank:
    // every mpi_* neighbour is MPI_PROC_NULL, so every taper strip is active).
    void init_geometry(int taper_width, T taper_slope) {
        pml = taper_width;
        alpha = taper_slope;
        const int nx_loc = nx - 1, ny_loc = ny - 1, nz_loc = nz - 1;
        jac = ext.dx_elm * ext.dy_elm * ext.dz_elm / T(8);
        x1 = coordinates_1d<T>(nx, N, ext.x_loc_min, ext.x_loc_max);
        y1 = coordinates_1d<T>(ny, N, ext.y_loc_min, ext.y_loc_max);
        z1 = coordinates_1d<T>(nz, N, ext.z_loc_max, ext.z_loc_min);  // r upside down :155-157
        std::vector<T> w = gll_weights<T>(N);
        std::vector<T> px(nloc, T(0)), py(nloc, T(0)), pz(nloc, T(0));
        r.assign(nloc, 0); sin_t.assign(nloc, 0); cot_t.assign(nloc, 0);
        r_sin.assign(nloc, 0); rr_sin.assign(nloc, 0); W.assign(nloc, 0); taper.assign(nloc, 0);
        // 1-D damping profiles :190-294
        std::vector<T> pxl((size_t)nx * P, T(0)), pyl((size_t)ny * P, T(0)), pzl((size_t)nz * P, T(0));
        for (int ex = 0; ex <= pml - 1; ++ex)
            for (int n = 0; n <= N; ++n) {
                T d = ext.x_loc_min + T(pml) * ext.dx_elm - x1[(size_t)ex * P + n];
                T q = d / (T(pml) * ext.dx_elm);
                pxl[(size_t)ex * P + n] = alpha * (q * q);
            }
        for (int ex = nx_loc - pml + 1; ex <= nx_loc; ++ex)
            for (int n = 0; n <= N; ++n) {
                T d = ext.x_loc_max - T(pml) * ext.dx_elm - x1[(size_t)ex * P + n];
                T q = d / (T(pml) * ext.dx_elm);
                pxl[(size_t)ex * P + n] = alpha * (q * q);
            }
        for (int ey = 0; ey <= pml - 1; ++ey)
            for (int n = 0; n <= N; ++n) {
                T d = ext.y_loc_min + T(pml) * ext.dy_elm - y1[(size_t)ey * P + n];
                T q = d / (T(pml) * ext.dy_elm);
                pyl[(size_t)ey * P + n] = alpha * (q * q);
            }
        for (int ey = ny_loc - pml + 1; ey <= ny_loc; ++ey)
            for (int n = 0; n <= N; ++n) {
                T d = ext.y_loc_max - T(pml) * ext.dy_elm - y1[(size_t)ey * P + n];
                T q = d / (T(pml) * ext.dy_elm);
                pyl[(size_t)ey * P + n] = alpha * (q * q);
            }
        for (int ez = nz_loc - pml + 1; ez <= nz_loc; ++ez)
            for (int n = 0; n <= N; ++n) {
                T d = ext.z_loc_min + T(pml) * ext.dz_elm - z1[(size_t)ez * P + n];
                T q = d / (T(pml) * ext.dz_elm);
                pzl[(size_t)ez * P + n] = alpha * (q * q);
            }
        for (int k = 0; k < P; ++k)
            for (int j = 0; j < P; ++j)
                for (int i = 0; i < P; ++i)
                    for (int ez = 0; ez < nz; ++ez)
                        for (int ey = 0; ey < ny; ++ey)
                            for (int ex = 0; ex < nx; ++ex) {
                                size_t a = I(E(ex, ey, ez), i, j, k);
                                T th = x1[(size_t)ex * P + i];
                                T rr = z1[(size_t)ez * P + k];
                                r[a] = rr;
                                sin_t[a] = std::sin(th);
                                cot_t[a] = std::cos(th) / std::sin(th);
                                r_sin[a] = rr * sin_t[a];
                                rr_sin[a] = rr * r_sin[a];
                                W[a] = w[i] * w[j] * w[k];
                                px[a] = pxl[(size_t)ex * P + i];
                                py[a] = pyl[(size_t)ey * P + j];
                                pz[a] = pzl[(size_t)ez * P + k];
                            }
        // The WHERE block at :297-304 writes `prof`, which :308 overwrites
        // before any read: it has no effect and is not restated.
        // Corner normalisation and taper :308-316.
        for (size_t a = 0; a < nloc; ++a) {
            T prof = px[a] + py[a] + pz[a];
            T qz = T(2) * pz[a] / (T(1) + prof / alpha);
            T qy = T(2) * py[a] / (T(1) + prof / alpha);
            T qx = T(2) * px[a] / (T(1) + prof / alpha);
            T p2 = qx + qy + qz;
            taper[a] = std::exp(-(T(0.1) * (p2 * p2)));
        }
    }

    // init_auxiliary_model_parameters: src/model_paras.F90:389-416.
    void init_aux() {
        two_mu.resize(nloc); kappa.resize(nloc); tau.resize(nloc); mu_tau.resize(nloc); MM.resize(nloc);
        rho.assign(nloc, T(0));
        visco = false;
        for (size_t a = 0; a < nloc; ++a)
            if (qq[a] != std::numeric_limits<T>::max()) visco = true;  // src/evolution.f90:70-74
        for (size_t a = 0; a < nloc; ++a) {
            two_mu[a] = T(2) * mu[a];
            kappa[a] = lambda[a] + T(2) * mu[a] / T(3);
            rho[a] = rhoinv[a] > T(0) ? T(1) / rhoinv[a] : T(0);
            tau[a] = T(6.0814) * std::pow(qq[a], T(-1.015));
            mu_tau[a] = (T(1) + tau[a]) * mu[a];
            MM[a] = -(jac * (r[a] * r[a]) * sin_t[a] * rho[a] * W[a]);
        }
        assemble_local(MM.data(), nx, ny, nz, N);
    }

    // kinetic_energy: src/elastic_vars.F90:218-246, the element-local sum in
    // the working precision, Fortran array order (one rank: the MPI_ALLREDUCE
    // sum is the identity).
    T kinetic_energy() const {
        T s = T(0);
        for (size_t a = 0; a < nloc; ++a)
            s += (vx[a] * vx[a] + vy[a] * vy[a] + vz[a] * vz[a]) * rr_sin[a] * rho[a] * W[a];
        return T(0.5) * jac * s;
    }

    void alloc_state() {
        for (auto *v : {&vx, &vy, &vz, &sx, &sy, &sz, &sxx, &sxy, &sxz, &syy, &syz, &szz, &exx, &eyy, &ezz, &exy,
                        &eyx, &exz, &ezx, &ezy, &eyz, &L, &txx, &txy, &txz, &tyy, &tyz, &tzz})
            v->assign(nloc, T(0));
        if (keep_du)
            for (auto *v : {&dxux, &dyuy, &dzuz, &dxuy, &dyux, &dxuz, &dzux, &dyuz, &dzuy}) v->assign(nloc, T(0));
        for (auto &s : src) s.assign(nloc, T(0));
        if (visco)
            for (auto &m : M)
                for (auto &mk : m) mk.assign(nloc, T(0));
    }

    // ses3d_evolution: src/evolution.f90:87-444.
    void evolution() {
        const T two = 2;
        // zero strain :126-128 and strain line contractions :130-159
        par_range<T>(nel, [&](size_t e0, size_t e1) {
            for (auto *v : {&exx, &eyy, &ezz, &exy, &eyx, &exz, &ezx, &ezy, &eyz})
                for (int p = 0; p < NP; ++p)
                    for (size_t e = e0; e < e1; ++e) (*v)[e + nel * p] = 0;
            for (int i = 0; i < P; ++i)
                for (int q = 0; q < P; ++q) {
                    T d3 = two * dl[q * P + i] / ext.dz_elm;
                    T d2 = two * dl[q * P + i] / ext.dy_elm;
                    T d1 = two * dl[q * P + i] / ext.dx_elm;
                    for (int b = 0; b < P; ++b)
                        for (int a = 0; a < P; ++a) {
                            // z-derivative: last index i <- q
                            size_t o = I(0, a, b, i), s = I(0, a, b, q);
                            for (size_t e = e0; e < e1; ++e) {
                                ezz[o + e] = ezz[o + e] + vz[s + e] * d3;
                                ezy[o + e] = ezy[o + e] + vy[s + e] * d3;
                                ezx[o + e] = ezx[o + e] + vx[s + e] * d3;
                            }
                            // y-derivative: middle index
                            o = I(0, a, i, b); s = I(0, a, q, b);
                            for (size_t e = e0; e < e1; ++e) {
                                eyy[o + e] = eyy[o + e] + vy[s + e] * d2;
                                eyx[o + e] = eyx[o + e] + vx[s + e] * d2;
                                eyz[o + e] = eyz[o + e] + vz[s + e] * d2;
                            }
                            // x-derivative: first GLL index
                            o = I(0, i, a, b); s = I(0, q, a, b);
                            for (size_t e = e0; e < e1; ++e) {
                                exx[o + e] = exx[o + e] + vx[s + e] * d1;
                                exy[o + e] = exy[o + e] + vy[s + e] * d1;
                                exz[o + e] = exz[o + e] + vz[s + e] * d1;
                            }
                        }
                }
            // spherical completion :165-173, symmetrisation :206-208,
            // stress rates :216-296, stress integration :306-311,
            // moment-tensor and single-force source superposition :315-325
            for (int p = 0; p < NP; ++p)
                for (size_t e = e0; e < e1; ++e) {
                    size_t a = e + nel * p;
                    T rr = r[a], rs = r_sin[a], ct = cot_t[a];
                    ezz[a] = -ezz[a];
                    eyy[a] = eyy[a] / rs + (vz[a] + vx[a] * ct) / rr;
                    exx[a] = (vz[a] + exx[a]) / rr;
                    ezx[a] = -ezx[a];
                    exz[a] = (exz[a] - vx[a]) / rr;
                    ezy[a] = -ezy[a];
                    eyz[a] = -vy[a] / rr + eyz[a] / rs;
                    exy[a] = exy[a] / rr;
                    eyx[a] = -(vy[a] * ct / rr) + eyx[a] / rs;
                    if (keep_du) {  // :179-187
                        dzuz[a] = dzuz[a] + dt * ezz[a];
                        dyuy[a] = dyuy[a] + dt * eyy[a];
                        dxux[a] = dxux[a] + dt * exx[a];
                        dzux[a] = dzux[a] + dt * ezx[a];
                        dxuz[a] = dxuz[a] + dt * exz[a];
                        dzuy[a] = dzuy[a] + dt * ezy[a];
                        dyuz[a] = dyuz[a] + dt * eyz[a];
                        dxuy[a] = dxuy[a] + dt * exy[a];
                        dyux[a] = dyux[a] + dt * eyx[a];
                    }
                    exy[a] = (exy[a] + eyx[a]) / two;
                    exz[a] = (exz[a] + ezx[a]) / two;
                    eyz[a] = (eyz[a] + ezy[a]) / two;
                    T s_xx, s_yy, s_zz, s_xy, s_xz, s_yz;
                    if (visco) {
                        T Mdx = M[0][0][a] + M[0][1][a] + M[0][2][a];
                        T Mdy = M[1][0][a] + M[1][1][a] + M[1][2][a];
                        T Mdz = M[2][0][a] + M[2][1][a] + M[2][2][a];
                        T Mdum = Mdx + Mdy + Mdz;
                        T Lv = (kappa[a] - two * mu_tau[a] / T(3)) * (exx[a] + eyy[a] + ezz[a]) -
                               two_mu[a] * Mdum / T(3);
                        L[a] = Lv;
                        s_xx = Lv + two * mu_tau[a] * exx[a] + two_mu[a] * Mdx + C[a] * ezz[a] + A[a] * (eyy[a] + exx[a]);
                        s_yy = Lv + two * mu_tau[a] * eyy[a] + two_mu[a] * Mdy + C[a] * ezz[a] + A[a] * (eyy[a] + exx[a]);
                        s_zz = Lv + two * mu_tau[a] * ezz[a] + two_mu[a] * Mdz + C[a] * (eyy[a] + exx[a]);
                        T Mxy = M[3][0][a] + M[3][1][a] + M[3][2][a];
                        T Mxz = M[4][0][a] + M[4][1][a] + M[4][2][a];
                        T Myz = M[5][0][a] + M[5][1][a] + M[5][2][a];
                        s_xy = two * mu_tau[a] * exy[a] + two_mu[a] * Mxy;
                        s_xz = two * mu_tau[a] * exz[a] + two_mu[a] * Mxz + two * B[a] * exz[a];
                        s_yz = two * mu_tau[a] * eyz[a] + two_mu[a] * Myz + two * B[a] * eyz[a];
                    } else {
                        T Lv = lambda[a] * (exx[a] + eyy[a] + ezz[a]);
                        L[a] = Lv;
                        s_xx = Lv + two_mu[a] * exx[a] + C[a] * ezz[a] + A[a] * (eyy[a] + exx[a]);
                        s_yy = Lv + two_mu[a] * eyy[a] + C[a] * ezz[a] + A[a] * (eyy[a] + exx[a]);
                        s_zz = Lv + two_mu[a] * ezz[a] + C[a] * (eyy[a] + exx[a]);
                        s_xy = two_mu[a] * exy[a];
                        s_xz = two_mu[a] * exz[a] + two * B[a] * exz[a];
                        s_yz = two_mu[a] * eyz[a] + two * B[a] * eyz[a];
                    }
                    sxx[a] = sxx[a] + dt * s_xx;
                    sxy[a] = sxy[a] + dt * s_xy;
                    sxz[a] = sxz[a] + dt * s_xz;
                    syy[a] = syy[a] + dt * s_yy;
                    syz[a] = syz[a] + dt * s_yz;
                    szz[a] = szz[a] + dt * s_zz;
                    txx[a] = sxx[a] + src[0][a];
                    txy[a] = sxy[a] + src[1][a];
                    txz[a] = sxz[a] + src[2][a];
                    tyy[a] = syy[a] + src[3][a];
                    tyz[a] = syz[a] + src[4][a];
                    tzz[a] = szz[a] + src[5][a];
                    sx[a] = src[6][a];
                    sy[a] = src[7][a];
                    sz[a] = src[8][a];
                }
            // weak form of the stress divergence :332-367
            std::vector<T> dxq(e1 - e0), dyq(e1 - e0), dzq(e1 - e0);
            for (int i = 0; i < P; ++i)
                for (int j = 0; j < P; ++j)
                    for (int k = 0; k < P; ++k) {
                        T d1 = (two / ext.dx_elm) * jac;
                        T d2 = (two / ext.dy_elm) * jac;
                        T d3 = -((two / ext.dz_elm) * jac);
                        size_t o = I(0, i, j, k);
                        for (int q = 0; q < P; ++q) {
                            size_t ax = I(0, q, j, k), ay = I(0, i, q, k), az = I(0, i, j, q);
                            for (size_t e = e0; e < e1; ++e) {
                                dxq[e - e0] = W[ax + e] * dl[i * P + q] * r_sin[ax + e] * d1;
                                dyq[e - e0] = W[ay + e] * dl[j * P + q] * r[ay + e] * d2;
                                dzq[e - e0] = W[az + e] * dl[k * P + q] * rr_sin[az + e] * d3;
                            }
                            for (size_t e = e0; e < e1; ++e) {
                                T gx = dxq[e - e0], gy = dyq[e - e0], gz = dzq[e - e0];
                                sx[o + e] = sx[o + e] + txz[az + e] * gz + txy[ay + e] * gy + txx[ax + e] * gx;
                                sy[o + e] = sy[o + e] + tyz[az + e] * gz + tyy[ay + e] * gy + txy[ax + e] * gx;
                                sz[o + e] = sz[o + e] + tzz[az + e] * gz + tyz[ay + e] * gy + txz[ax + e] * gx;
                            }
                        }
                    }
            // divide by the assembled mass matrix :372-374
            for (int p = 0; p < NP; ++p)
                for (size_t e = e0; e < e1; ++e) {
                    size_t a = e + nel * p;
                    sx[a] = sx[a] / MM[a];
                    sy[a] = sy[a] / MM[a];
                    sz[a] = sz[a] / MM[a];
                }
        });
        // local assembly :379-381 (the global exchange :386-388 is a no-op on one rank)
        assemble_local(sx.data(), nx, ny, nz, N);
        assemble_local(sy.data(), nx, ny, nz, N);
        assemble_local(sz.data(), nx, ny, nz, N);
        // velocity update :393-395, taper :400-409, memory variables :415-442
        par_range<T>(nloc, [&](size_t a0, size_t a1) {
            for (size_t a = a0; a < a1; ++a) {
                vx[a] = vx[a] + dt * sx[a];
                vy[a] = vy[a] + dt * sy[a];
                vz[a] = vz[a] + dt * sz[a];
                vx[a] = vx[a] * taper[a];
                vy[a] = vy[a] * taper[a];
                vz[a] = vz[a] * taper[a];
                sxx[a] = sxx[a] * taper[a];
                sxy[a] = sxy[a] * taper[a];
                sxz[a] = sxz[a] * taper[a];
                syy[a] = syy[a] * taper[a];
                syz[a] = syz[a] * taper[a];
                szz[a] = szz[a] * taper[a];
                if (visco) {
                    const T *e6[6] = {&exx[a], &eyy[a], &ezz[a], &exy[a], &exz[a], &eyz[a]};
                    for (int k = 0; k < nrdiss; ++k) {
                        T Lk = dt * tau[a] / (T(nrdiss) * tau_p[k]);
                        for (int c = 0; c < 6; ++c) {
                            T m = M[c][k][a];
                            M[c][k][a] = m - dt * m / tau_p[k] - Lk * (*e6[c]);
                        }
                    }
                }
            }
        });
    }

    // channel add_m**/add_f*: src/config/channel_mod.f90:859-1095 (assigning
    // one element slab; slabs persist until reassigned).
    void add_sources(int it_) {
        for (auto &s : sources) {
            size_t e = E(s.ex, s.ey, s.ez);
            for (auto &c : s.ch) {
                T d = c.data[it_ - 1];
                for (int p = 0; p < NP; ++p) {
                    size_t a = e + nel * p;
                    if (c.comp < 6)
                        src[c.comp][a] = -d * s.vm[p] / (jac * W[a] * rr_sin[a]);
                    else
                        src[c.comp][a] = -d * s.vm[p];
                }
            }
        }
    }

    // Rotation rates as get_field / record_rot_v* evaluate them after a step
    // (src/volume_snapshot.f90:238-246, src/config/channel_mod.f90:620-812).
    T rot(int c, size_t a) const {
        if (c == 0) return -vy[a] / r[a] + eyz[a] / r_sin[a] + ezy[a];
        if (c == 1) return -ezx[a] + (vx[a] - exz[a]) / r[a];
        return (exy[a] + vy[a] * cot_t[a] - eyx[a] / sin_t[a]) / r[a];
    }

    // record_vx/vy/vz (src/config/channel_mod.f90:505-592), record_n
    // (:532-540), record_rot_v* (:620-712), record_m** / record_f*
    // (:859-1095): SUM over the element of vanderm times the quantity.
    void record(int it_) {
        for (auto &rc : receivers) {
            size_t e = E(rc.ex, rc.ey, rc.ez);
            const std::vector<T> *v3[3] = {&vx, &vy, &vz};
            for (int c = 0; c < 3; ++c) {
                T s = 0;
                for (int p = 0; p < NP; ++p) s = s + rc.vm[p] * (*v3[c])[e + nel * p];
                rc.data[c][it_ - 1] = s;
            }
            for (int b = 3; b < 16; ++b) {
                if (!((rc.mask >> b) & 1u)) continue;
                T s = 0;
                for (int p = 0; p < NP; ++p) {
                    const size_t a = e + nel * p;
                    T q;
                    if (b == 3) q = T(-1) * rc.vm[p] * vx[a];
                    else if (b <= 6) q = rc.vm[p] * rot(b - 4, a);
                    else q = rc.vm[p] * src[b - 7][a];
                    s = s + q;
                }
                rc.data[b][it_ - 1] = s;
            }
        }
    }

    // cfl_loc (src/model_paras.F90:529-561) and f_c_loc (:464-494) on the
    // rank-6 fields, with cp/cs from init_auxiliary_model_parameters (:402-403).
    void courant(T out[2]) const {
        std::vector<T> cp(nloc), cs(nloc), th(nloc), ph(nloc);
        for (int k = 0; k < P; ++k)
            for (int j = 0; j < P; ++j)
                for (int i = 0; i < P; ++i)
                    for (int ez = 0; ez < nz; ++ez)
                        for (int ey = 0; ey < ny; ++ey)
                            for (int ex = 0; ex < nx; ++ex) {
                                size_t a = I(E(ex, ey, ez), i, j, k);
                                cp[a] = std::sqrt((lambda[a] + T(2) * mu[a]) * rhoinv[a]);
                                cs[a] = std::sqrt(mu[a] * rhoinv[a]);
                                th[a] = x1[(size_t)ex * P + i];
                                ph[a] = y1[(size_t)ey * P + j];
                            }
        T cfl[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (size_t e = 0; e < nel; ++e)
            for (int k = 0; k < P; ++k)
                for (int j = 0; j < P; ++j)
                    for (int i = 0; i < P; ++i) {
                        size_t a = I(e, i, j, k);
                        T vmax = (cs[a] < cp[a]) ? cp[a] : cs[a];  // MERGE(cp, cs, cs < cp)
                        if (i >= 1) cfl[0] = std::max(cfl[0], vmax / (r[a] * (th[a] - th[I(e, i - 1, j, k)])));
                        if (j >= 1) cfl[1] = std::max(cfl[1], vmax / (r_sin[a] * (ph[a] - ph[I(e, i, j - 1, k)])));
                        if (k >= 1) cfl[2] = std::max(cfl[2], vmax / (r[I(e, i, j, k - 1)] - r[a]));
                    }
        T fc[3] = {INFINITY, INFINITY, INFINITY};
        const T s = 2;
        for (size_t e = 0; e < nel; ++e)
            for (int b = 0; b < P; ++b)
                for (int c = 0; c < P; ++c) {
                    T sx = 0, sy = 0, sz = 0;
                    for (int q = 0; q < P; ++q) {
                        size_t ax = I(e, q, b, c), ay = I(e, b, q, c), az = I(e, b, c, q);
                        sx = sx + ((cs[ax] > cp[ax]) ? cp[ax] : cs[ax]);
                        sy = sy + ((cs[ay] > cp[ay]) ? cp[ay] : cs[ay]);
                        sz = sz + ((cs[az] > cp[az]) ? cp[az] : cs[az]);
                    }
                    T vx = sx / T(P), vy = sy / T(P), vz = sz / T(P);
                    T arcx = r[I(e, 0, b, c)] * ext.dx_elm;
                    T arcy = r_sin[I(e, b, 0, c)] * ext.dy_elm;
                    if (vx > 0) fc[0] = std::min(fc[0], vx / s / arcx);
                    if (vy > 0) fc[1] = std::min(fc[1], vy / s / arcy);
                    if (vz > 0) fc[2] = std::min(fc[2], vz / s / ext.dz_elm);
                }
        out[0] = std::max(cfl[0] * dt, std::max(cfl[1] * dt, cfl[2] * dt));
        out[1] = std::min(fc[0], std::min(fc[1], fc[2]));
    }

    // Forward loop: src/ses3d-nt.F90:240-270.
    void run(int nsteps) {
        for (int n = 0; n < nsteps; ++n) {
            ++it;
            evolution();
            add_sources(it);
            record(it);
        }
    }
};

struct Handle {
    int precision;
    void *sim;
};

template <class T>
Sim<T> *S(Handle *h) { return static_cast<Sim<T> *>(h->sim); }

}  // namespace

extern "C" {

struct oracle_cfg {
    int nx, ny, nz, lpd, taper_width, nt, precision;
    float taper_slope, lat_min, lat_max, lon_min, lon_max, rad_min, rad_max, dt;
};

int oracle_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// GLL tables in float: knots[lpd+1], weights[lpd+1], dl[(lpd+1)^2] (dl[i*(lpd+1)+j]).
int oracle_gll_size(int lpd) { return (int)gll_knots<float>(lpd).size() * 1000 + (int)gll_weights<float>(lpd).size(); }

void oracle_gll_f32(int lpd, float *knots, float *weights, float *dl) {
    auto k = gll_knots<float>(lpd);
    auto w = gll_weights<float>(lpd);
    for (size_t i = 0; i < k.size(); ++i) {
        knots[i] = k[i];
        weights[i] = w[i];
    }
    for (int i = 0; i <= lpd; ++i)
        for (int j = 0; j <= lpd; ++j) dl[i * (lpd + 1) + j] = get_dlgll<float>(lpd, i, j);
}

void oracle_gll_f64(int lpd, double *knots, double *weights, double *dl) {
    auto k = gll_knots<double>(lpd);
    auto w = gll_weights<double>(lpd);
    for (size_t i = 0; i < k.size(); ++i) {
        knots[i] = k[i];
        weights[i] = w[i];
    }
    for (int i = 0; i <= lpd; ++i)
        for (int j = 0; j <= lpd; ++j) dl[i * (lpd + 1) + j] = get_dlgll<double>(lpd, i, j);
}

void oracle_coordinates_1d(int elms, int lpd, float mn, float mx, float *out) {
    auto c = coordinates_1d<float>(elms, lpd, mn, mx);
    std::memcpy(out, c.data(), c.size() * sizeof(float));
}

void oracle_lagrange(float x, int n, const float *knots, float *out) {
    std::vector<float> k(knots, knots + n);
    auto l = lagrange<float>(x, k);
    std::memcpy(out, l.data(), n * sizeof(float));
}

void oracle_assemble_f32(int nx, int ny, int nz, int lpd, float *field) { assemble_local<float>(field, nx, ny, nz, lpd); }
void oracle_assemble_f64(int nx, int ny, int nz, int lpd, double *field) { assemble_local<double>(field, nx, ny, nz, lpd); }

void oracle_stf(int kind, float onset, float width, float dt, int nt, float *out) {
    source_signature<float>(kind, onset, width, dt, nt, out);
}

void *oracle_create(const oracle_cfg *c) {
    Handle *h = new Handle{c->precision, nullptr};
    auto make = [&](auto tag) {
        using T = decltype(tag);
        auto *s = new Sim<T>();
        s->nx = c->nx; s->ny = c->ny; s->nz = c->nz; s->N = c->lpd; s->P = c->lpd + 1;
        s->NP = s->P * s->P * s->P; s->nt = c->nt;
        s->nel = (size_t)c->nx * c->ny * c->nz;
        s->nloc = s->nel * s->NP;
        s->dt = T(c->dt);
        s->ext = make_extents<T>(c->nx, c->ny, c->nz, T(c->lat_min), T(c->lat_max), T(c->lon_min), T(c->lon_max),
                                 T(c->rad_min), T(c->rad_max));
        s->dl.resize((size_t)s->P * s->P);
        for (int i = 0; i < s->P; ++i)
            for (int j = 0; j < s->P; ++j) s->dl[i * s->P + j] = get_dlgll<T>(s->N, i, j);
        s->init_geometry(c->taper_width, T(c->taper_slope));
        return (void *)s;
    };
    h->sim = (c->precision == 8) ? make(double(0)) : make(float(0));
    return h;
}

// Model arrays in the reference raw layout (Fortran order rank 6), float32 as
// read by src/model_paras.F90:97-137. NULL a/b/c mean zero, NULL q means HUGE.
int oracle_set_model(void *hv, const float *rhoinv, const float *lambda, const float *mu, const float *a,
                     const float *b, const float *c, const float *q) {
    Handle *h = (Handle *)hv;
    auto go = [&](auto *s) {
        using T = typename std::remove_pointer_t<decltype(s)>::real_t;
        size_t n = s->nloc;
        auto cp = [&](std::vector<T> &dst, const float *src, T dflt) {
            dst.resize(n);
            for (size_t i = 0; i < n; ++i) dst[i] = src ? T(src[i]) : dflt;
        };
        cp(s->rhoinv, rhoinv, 0); cp(s->lambda, lambda, 0); cp(s->mu, mu, 0);
        cp(s->A, a, 0); cp(s->B, b, 0); cp(s->C, c, 0);
        s->qq.resize(n);
        for (size_t i = 0; i < n; ++i)
            s->qq[i] = q ? (q[i] == std::numeric_limits<float>::max() ? std::numeric_limits<T>::max() : T(q[i]))
                         : std::numeric_limits<T>::max();
        s->init_aux();
        s->alloc_state();
        return 0;
    };
    if (h->precision == 8) return go(S<double>(h));
    return go(S<float>(h));
}

// construct_point_cls: src/config/point.f90:150-254 with std_x/y/z :553-657,
// elm_*_loc :826-889, in_domain/in_rank :735-803 and the Vandermonde matrix of
// src/interpolation_mod.f90:194-205. Always float32 as in the reference.
// Returns 0 on success, -1 invalid coordinates, -2 outside the domain.
int oracle_locate_cfg(const oracle_cfg *c, float lat, float lon, float depth, int *exyz, float *vm) {
    typedef float T;
    if (!(std::fabs(lat) <= T(90)) || !(std::fabs(lon) <= T(180)) || !(T(0) <= depth && depth < T(6371000.0)))
        return -1;
    Extents<T> e = make_extents<T>(c->nx, c->ny, c->nz, c->lat_min, c->lat_max, c->lon_min, c->lon_max, c->rad_min,
                                   c->rad_max);
    T x = deg2rad<T>(T(90) - lat);
    T y = deg2rad<T>(lon);
    T z = T(6371000.0) - depth;
    if (!(e.x_glb_min < x && x < e.x_glb_max && e.y_glb_min < y && y < e.y_glb_max && e.z_glb_min < z &&
          z <= e.z_glb_max))
        return -2;
    if (!(e.x_loc_min < x && x <= e.x_loc_max && e.y_loc_min < y && y <= e.y_loc_max && e.z_loc_min < z &&
          z <= e.z_loc_max))
        return -2;
    int ex = (c->nx - 1) - (int)std::floor((e.x_loc_max - x) / e.dx_elm);
    int ey = (c->ny - 1) - (int)std::floor((e.y_loc_max - y) / e.dy_elm);
    int ez = (int)std::floor((e.z_loc_max - z) / e.dz_elm);
    T sx = T(2) * ((x - e.x_loc_min) / e.dx_elm - T(ex)) - T(1);
    T sy = T(2) * ((y - e.y_loc_min) / e.dy_elm - T(ey)) - T(1);
    T sz = T(2) * ((e.z_loc_max - z) / e.dz_elm - T(ez)) - T(1);
    auto knots = gll_knots<T>(c->lpd);
    auto lx = lagrange<T>(sx, knots), ly = lagrange<T>(sy, knots), lz = lagrange<T>(sz, knots);
    int P = c->lpd + 1;
    exyz[0] = ex; exyz[1] = ey; exyz[2] = ez;
    for (int k = 0; k < P; ++k)
        for (int j = 0; j < P; ++j)
            for (int i = 0; i < P; ++i) vm[i + P * (j + P * k)] = lx[i] * ly[j] * lz[k];
    return 0;
}

// create_from_source_mt (src/config/source.f90:274-327): channels mxx..mzz
// with data = stf*M_c, all-zero channels dropped. kind 1 is
// create_from_source_sf (:215-258): channels fx, fy, fz, all kept.
int oracle_add_source(void *hv, int ex, int ey, int ez, const float *vm, int kind, const float *comp,
                      const float *stf) {
    Handle *h = (Handle *)hv;
    auto go = [&](auto *s) {
        using T = typename std::remove_pointer_t<decltype(s)>::real_t;
        typename std::remove_pointer_t<decltype(s)>::Source src;
        src.ex = ex; src.ey = ey; src.ez = ez;
        src.vm.assign(vm, vm + s->NP);
        int nc = kind == 0 ? 6 : 3;
        for (int c = 0; c < nc; ++c) {
            typename std::remove_pointer_t<decltype(s)>::Channel ch;
            ch.comp = kind == 0 ? c : 6 + c;
            ch.data.resize(s->nt);
            bool nz = false;
            for (int i = 0; i < s->nt; ++i) {
                float d = stf[i] * comp[c];  // data*moment_tensor(c) in REAL32
                ch.data[i] = T(d);
                if (d != 0.0f) nz = true;
            }
            if (kind == 0 && !nz) continue;
            src.ch.push_back(std::move(ch));
        }
        s->sources.push_back(std::move(src));
        return 0;
    };
    if (h->precision == 8) return go(S<double>(h));
    return go(S<float>(h));
}

// Receiver with a channel mask (bits as the GPU library's SESNT_CH_*: vx vy
// vz n rot_vx rot_vy rot_vz mxx mxy mxz myy myz mzz fx fy fz).
int oracle_add_receiver_mask(void *hv, int ex, int ey, int ez, const float *vm, unsigned mask) {
    Handle *h = (Handle *)hv;
    auto go = [&](auto *s) {
        typename std::remove_pointer_t<decltype(s)>::Receiver rc;
        rc.ex = ex; rc.ey = ey; rc.ez = ez;
        rc.mask = mask | 7u;
        rc.vm.assign(vm, vm + s->NP);
        for (auto &d : rc.data) d.assign(s->nt, 0);
        s->receivers.push_back(std::move(rc));
        return 0;
    };
    if (h->precision == 8) return go(S<double>(h));
    return go(S<float>(h));
}

int oracle_add_receiver(void *hv, int ex, int ey, int ez, const float *vm) {
    return oracle_add_receiver_mask(hv, ex, ey, ez, vm, 7u);
}

// Keep the displacement gradient (call before oracle_set_model).
void oracle_keep_strain(void *hv) {
    Handle *h = (Handle *)hv;
    if (h->precision == 8) S<double>(h)->keep_du = true;
    else S<float>(h)->keep_du = true;
}

// One receiver channel (bit b of the mask), [nt] in the working precision.
int oracle_get_trace(void *hv, int receiver, int bit, void *out) {
    Handle *h = (Handle *)hv;
    auto go = [&](auto *s) {
        using T = typename std::remove_pointer_t<decltype(s)>::real_t;
        if (receiver < 0 || receiver >= (int)s->receivers.size() || bit < 0 || bit > 15) return -1;
        const auto &rc = s->receivers[receiver];
        if (!((rc.mask >> bit) & 1u)) return -1;
        std::memcpy(out, rc.data[bit].data(), s->nt * sizeof(T));
        return 0;
    };
    if (h->precision == 8) return go(S<double>(h));
    return go(S<float>(h));
}

int oracle_run(void *hv, int nsteps) {
    Handle *h = (Handle *)hv;
    if (h->precision == 8) S<double>(h)->run(nsteps);
    else S<float>(h)->run(nsteps);
    return 0;
}

// which: 0..2 vx,vy,vz; 3..8 sxx,sxy,sxz,syy,syz,szz; 9 taper; 10 MM
// (assembled); 11 r; 12 sin_theta; 13..30 memory variables (comp*3+k);
// 31..39 exx,eyy,ezz,exy,exz,eyz,eyx,ezx,ezy (last step's strain rates);
// get_field of src/volume_snapshot.f90:192-298: 40 pressure, 41..46 exx exy
// exz eyy eyz ezz (displacement gradient), 47..49 rot_vx rot_vy rot_vz, 50..54
// lambda mu a b c.
int oracle_get_field(void *hv, int which, void *out) {
    Handle *h = (Handle *)hv;
    auto go = [&](auto *s) {
        using T = typename std::remove_pointer_t<decltype(s)>::real_t;
        const std::vector<T> *f = nullptr;
        std::vector<T> tmp;
        if (which >= 40 && which <= 49) {
            if (which >= 41 && which <= 46 && !s->keep_du) return -1;
            tmp.resize(s->nloc);
            for (size_t a = 0; a < s->nloc; ++a) {
                T x;
                switch (which) {
                    case 40: x = T(-1) * (s->sxx[a] + s->syy[a] + s->szz[a]) / T(3); break;
                    case 41: x = s->dxux[a]; break;
                    case 42: x = (s->dxuy[a] + s->dyux[a]) / T(2); break;
                    case 43: x = (s->dxuz[a] + s->dzux[a]) / T(2); break;
                    case 44: x = s->dyuy[a]; break;
                    case 45: x = (s->dyuz[a] + s->dzuy[a]) / T(2); break;
                    case 46: x = s->dzuz[a]; break;
                    default: x = s->rot(which - 47, a);
                }
                tmp[a] = x;
            }
            f = &tmp;
        }
        switch (which) {
            case 50: f = &s->lambda; break; case 51: f = &s->mu; break;
            case 52: f = &s->A; break; case 53: f = &s->B; break; case 54: f = &s->C; break;
            case 0: f = &s->vx; break; case 1: f = &s->vy; break; case 2: f = &s->vz; break;
            case 3: f = &s->sxx; break; case 4: f = &s->sxy; break; case 5: f = &s->sxz; break;
            case 6: f = &s->syy; break; case 7: f = &s->syz; break; case 8: f = &s->szz; break;
            case 9: f = &s->taper; break; case 10: f = &s->MM; break; case 11: f = &s->r; break;
            case 12: f = &s->sin_t; break;
            case 31: f = &s->exx; break; case 32: f = &s->eyy; break; case 33: f = &s->ezz; break;
            case 34: f = &s->exy; break; case 35: f = &s->exz; break; case 36: f = &s->eyz; break;
            case 37: f = &s->eyx; break; case 38: f = &s->ezx; break; case 39: f = &s->ezy; break;
            default:
                if (which >= 13 && which < 31 && s->visco) f = &s->M[(which - 13) / 3][(which - 13) % 3];
        }
        if (!f || f->empty()) return -1;
        std::memcpy(out, f->data(), f->size() * sizeof(T));
        return 0;
    };
    if (h->precision == 8) return go(S<double>(h));
    return go(S<float>(h));
}

// Seismograms [nrec][3][nt] (vx, vy, vz).
int oracle_get_seismograms(void *hv, void *out) {
    Handle *h = (Handle *)hv;
    auto go = [&](auto *s) {
        using T = typename std::remove_pointer_t<decltype(s)>::real_t;
        T *o = (T *)out;
        for (auto &rc : s->receivers)
            for (int c = 0; c < 3; ++c) {
                std::memcpy(o, rc.data[c].data(), s->nt * sizeof(T));
                o += s->nt;
            }
        return 0;
    };
    if (h->precision == 8) return go(S<double>(h));
    return go(S<float>(h));
}

int oracle_courant(void *hv, float out[2]) {
    Handle *h = (Handle *)hv;
    if (h->precision == 8) {
        double o[2];
        S<double>(h)->courant(o);
        out[0] = (float)o[0];
        out[1] = (float)o[1];
    } else {
        S<float>(h)->courant(out);
    }
    return 0;
}

int oracle_kinetic_energy(void *hv, double *out) {
    Handle *h = (Handle *)hv;
    *out = h->precision == 8 ? S<double>(h)->kinetic_energy() : (double)S<float>(h)->kinetic_energy();
    return 0;
}

int oracle_is_visco(void *hv) {
    Handle *h = (Handle *)hv;
    return h->precision == 8 ? S<double>(h)->visco : S<float>(h)->visco;
}

void oracle_destroy(void *hv) {
    Handle *h = (Handle *)hv;
    if (!h) return;
    if (h->precision == 8) delete S<double>(h);
    else delete S<float>(h);
    delete h;
}

}  // extern "C"
