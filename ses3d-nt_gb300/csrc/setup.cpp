// Host-side set-up for the GB300 time step: GLL tables, domain extents,
// element coordinates, taper profiles, point location and source-time
// functions. Compiled with -ffp-contract=off so the float32 routines round
// exactly like the reference's REAL32 code on both x86-64 and aarch64.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sesnt_internal.h"

namespace sesnt {

namespace {

template <typename T>
T pi_val() {
    return T(2) * std::acos(T(0));  // src/parameters.F90:67 (2*ACOS(0) in the working kind)
}

template <typename T>
T to_radians(T deg) {
    return deg * pi_val<T>() / T(180);  // src/misc/coordinate_utilities_mod.f90:79-82
}

}  // namespace

// GLL points for lpd 1..7. The closed forms for lpd <= 6 and the 16-digit
// values for lpd 7 are the published Gauss-Lobatto-Legendre nodes, written as
// the reference tabulates them (src/gll_mod.f90:61-135) so the float32 values
// agree bit for bit.
template <typename T>
std::vector<T> gll_points(int lpd) {
    std::vector<T> x;
    if (lpd < 1) return x;
    x.assign(lpd + 1, T(0));
    x.front() = T(-1);
    x.back() = T(1);
    auto mirror = [&](T inner_a, T inner_b) {  // fill symmetric interior points
        std::vector<T> in = {inner_a, inner_b};
        int m = (lpd - 1) / 2;
        for (int q = 0; q < m; ++q) {
            x[1 + q] = -in[q];
            x[lpd - 1 - q] = in[q];
        }
    };
    switch (lpd) {
        case 1: case 2: break;
        case 3: mirror(std::sqrt(T(1) / T(5)), T(0)); break;
        case 4: mirror(std::sqrt(T(3) / T(7)), T(0)); break;
        case 5: {
            T r7 = std::sqrt(T(7)), r21 = std::sqrt(T(21));
            mirror(std::sqrt(T(2) * r7 + T(7)) / r21, std::sqrt(T(7) - T(2) * r7) / r21);
        } break;
        case 6: {
            T r15 = std::sqrt(T(15)), r33 = std::sqrt(T(33));
            mirror(std::sqrt(T(2) * r15 + T(15)) / r33, std::sqrt(T(15) - T(2) * r15) / r33);
        } break;
        case 7: {
            const T v[3] = {T(0.8717401485096066), T(0.5917001814331423), T(0.2092992179024789)};
            for (int q = 0; q < 3; ++q) {
                x[1 + q] = -v[q];
                x[6 - q] = v[q];
            }
        } break;
        default: std::fill(x.begin(), x.end(), T(0)); break;
    }
    return x;
}

// GLL quadrature weights, src/gll_mod.f90:66-165.
template <typename T>
std::vector<T> gll_quadrature_weights(int lpd) {
    std::vector<T> w;
    if (lpd < 1) return w;
    w.assign(lpd + 1, T(0));
    auto sym = [&](std::initializer_list<T> half) {
        int q = 0;
        for (T v : half) {
            w[q] = v;
            w[lpd - q] = v;
            ++q;
        }
    };
    switch (lpd) {
        case 1: sym({T(0.5)}); break;
        case 2: sym({T(1) / T(3), T(4) / T(3)}); break;
        case 3: sym({T(1) / T(6), T(5) / T(6)}); break;
        case 4: sym({T(1) / T(10), T(49) / T(90), T(32) / T(45)}); break;
        case 5: {
            T r7 = std::sqrt(T(7));
            sym({T(1) / T(15), T(63) / (T(10) * r7 + T(140)), -T(63) / (T(10) * r7 - T(140))});
        } break;
        case 6: {
            T r15 = std::sqrt(T(15));
            sym({T(1) / T(21), T(14641) / (T(2450) * r15 + T(43400)), -T(14641) / (T(2450) * r15 - T(43400)),
                 T(256) / T(525)});
        } break;
        case 7:
            sym({T(0.0357142857142857), T(0.2107042271435061), T(0.3411226924835044), T(0.4124587946587038)});
            break;
        default: break;
    }
    return w;
}

// d[i*P+j] = derivative of the i-th Lagrange polynomial at point j
// (src/gll_mod.f90:251-275): for i == j the sum of 1/(x_i - x_m) over the
// other points, otherwise prod_{m != i,j}(x_j - x_m) / prod_{m != i}(x_i - x_m),
// accumulated in index order.
template <typename T>
std::vector<T> lagrange_derivative_matrix(int lpd) {
    std::vector<T> x = gll_points<T>(lpd);
    const int P = lpd + 1;
    std::vector<T> d((size_t)P * P, T(0));
    for (int i = 0; i < P; ++i)
        for (int j = 0; j < P; ++j) {
            if (i == j) {
                T acc = 0;
                for (int m = 0; m < P; ++m)
                    if (x[m] != x[i]) acc = acc + T(1) / (x[i] - x[m]);
                d[i * P + j] = acc;
            } else {
                T num = 1, den = 1;
                for (int m = 0; m < P; ++m) {
                    if (x[m] == x[i]) continue;
                    if (x[m] != x[j]) num = num * (x[j] - x[m]);
                    den = den * (x[i] - x[m]);
                }
                d[i * P + j] = num / den;
            }
        }
    return d;
}

// Domain extents of the single partition (src/config/model.f90:90-237 with
// one rank: the local bounds are the global minimum plus zero or one global
// extent, which the reference uses instead of the global maximum).
template <typename T>
Domain<T> make_domain(int nx, int ny, int nz, float lat_min, float lat_max, float lon_min, float lon_max,
                      float rad_min, float rad_max) {
    Domain<T> d;
    d.x_glb_min = to_radians<T>(T(90) - T(lat_max));
    d.x_glb_max = to_radians<T>(T(90) - T(lat_min));
    d.y_glb_min = to_radians<T>(T(lon_min));
    d.y_glb_max = to_radians<T>(T(lon_max));
    d.z_glb_min = T(rad_min);
    d.z_glb_max = T(rad_max);
    const T ext_x = d.x_glb_max - d.x_glb_min;
    const T ext_y = d.y_glb_max - d.y_glb_min;
    const T ext_z = d.z_glb_max - d.z_glb_min;
    d.dx_elm = ext_x / T(nx);
    d.dy_elm = ext_y / T(ny);
    d.dz_elm = ext_z / T(nz);
    d.x_loc_min = d.x_glb_min + T(0) * ext_x;
    d.x_loc_max = d.x_glb_min + T(1) * ext_x;
    d.y_loc_min = d.y_glb_min + T(0) * ext_y;
    d.y_loc_max = d.y_glb_min + T(1) * ext_y;
    d.z_loc_min = d.z_glb_min + T(0) * ext_z;
    d.z_loc_max = d.z_glb_min + T(1) * ext_z;
    return d;
}

// Element coordinates, src/coordinates_mod.f90:114-141: lo + (e + xi01)*delta
// with the last point pinned to hi, so shared element faces get identical
// coordinates.
template <typename T>
std::vector<T> element_coordinates(int elms, int lpd, T lo, T hi) {
    std::vector<T> xi = gll_points<T>(lpd);
    const int P = lpd + 1;
    for (T &v : xi) v = T(0.5) * (T(1) + v);
    const T delta = (hi - lo) / T(elms);
    std::vector<T> c((size_t)elms * P);
    for (int e = 0; e < elms; ++e)
        for (int n = 0; n < P; ++n) c[(size_t)e * P + n] = lo + (T(e) + xi[n]) * delta;
    c.back() = hi;
    return c;
}

// Quadratic damping profiles of the absorbing taper, src/geometric_paras.f90:190-294:
// alpha*((edge -/+ width*d_elm - x)/(width*d_elm))^2 inside the strips of
// `width` elements along the theta and phi sides and the bottom; the free
// surface (top) has none.
template <typename T>
void taper_profiles(int nx, int ny, int nz, int lpd, int width, T alpha, const Domain<T> &d, std::vector<T> &px,
                    std::vector<T> &py, std::vector<T> &pz) {
    const int P = lpd + 1;
    std::vector<T> x = element_coordinates<T>(nx, lpd, d.x_loc_min, d.x_loc_max);
    std::vector<T> y = element_coordinates<T>(ny, lpd, d.y_loc_min, d.y_loc_max);
    std::vector<T> z = element_coordinates<T>(nz, lpd, d.z_loc_max, d.z_loc_min);
    px.assign((size_t)nx * P, T(0));
    py.assign((size_t)ny * P, T(0));
    pz.assign((size_t)nz * P, T(0));
    auto strip = [&](std::vector<T> &prof, const std::vector<T> &c, int e0, int e1, T edge, T span) {
        for (int e = e0; e <= e1; ++e)
            for (int n = 0; n < P; ++n) {
                T q = (edge - c[(size_t)e * P + n]) / span;
                prof[(size_t)e * P + n] = alpha * (q * q);
            }
    };
    const T wx = T(width) * d.dx_elm, wy = T(width) * d.dy_elm, wz = T(width) * d.dz_elm;
    strip(px, x, 0, width - 1, d.x_loc_min + wx, wx);
    strip(px, x, nx - width, nx - 1, d.x_loc_max - wx, wx);
    strip(py, y, 0, width - 1, d.y_loc_min + wy, wy);
    strip(py, y, ny - width, ny - 1, d.y_loc_max - wy, wy);
    strip(pz, z, nz - width, nz - 1, d.z_loc_min + wz, wz);
}

namespace {

// Lagrange basis at x (src/interpolation_mod.f90:83-171): barycentric form
// prod(x - x_m)/(x - x_j) * w_j with w_j = 1/(prod_{m<j} * prod_{m>j}), and
// the exact Kronecker delta when x hits a point.
std::vector<float> lagrange_basis(float x, const std::vector<float> &pts) {
    const size_t n = pts.size();
    std::vector<float> l(n, 1.0f);
    if (n <= 1) return l;
    bool hit = false;
    for (float p : pts) hit = hit || !(x != p);
    if (hit) {
        for (size_t j = 0; j < n; ++j) l[j] = (x != pts[j]) ? 0.0f : 1.0f;
        return l;
    }
    float all = 1.0f;
    for (float p : pts) all = all * (x - p);
    for (size_t j = 0; j < n; ++j) {
        float lo = 1.0f, hi = 1.0f;
        for (size_t m = 0; m < j; ++m) lo = lo * (pts[j] - pts[m]);
        for (size_t m = j + 1; m < n; ++m) hi = hi * (pts[j] - pts[m]);
        float wj = 1.0f / (lo * hi);
        l[j] = all / (x - pts[j]) * wj;
    }
    return l;
}

}  // namespace

// Point location in float32, src/config/point.f90:150-254 (checks), :735-803
// (domain tests), :826-889 (element index), :553-657 (reference coordinate).
int locate_point(int nx, int ny, int nz, int lpd, float lat_min, float lat_max, float lon_min, float lon_max,
                 float rad_min, float rad_max, float lat, float lon, float depth, int elem[3], float *vanderm,
                 std::string &why) {
    const float earth_radius = 6371000.0f;  // src/parameters.F90:64
    if (!(std::fabs(lat) <= 90.0f) || !(std::fabs(lon) <= 180.0f) || !(0.0f <= depth && depth < earth_radius)) {
        why = "invalid latitude, longitude or depth";
        return -1;
    }
    Domain<float> d = make_domain<float>(nx, ny, nz, lat_min, lat_max, lon_min, lon_max, rad_min, rad_max);
    const float x = to_radians<float>(90.0f - lat);
    const float y = to_radians<float>(lon);
    const float z = earth_radius - depth;
    const bool in_domain = d.x_glb_min < x && x < d.x_glb_max && d.y_glb_min < y && y < d.y_glb_max &&
                           d.z_glb_min < z && z <= d.z_glb_max;
    const bool in_part = d.x_loc_min < x && x <= d.x_loc_max && d.y_loc_min < y && y <= d.y_loc_max &&
                         d.z_loc_min < z && z <= d.z_loc_max;
    if (!in_domain || !in_part) {
        why = "point not in the computational domain";
        return -2;
    }
    const int ex = (nx - 1) - (int)std::floor((d.x_loc_max - x) / d.dx_elm);
    const int ey = (ny - 1) - (int)std::floor((d.y_loc_max - y) / d.dy_elm);
    const int ez = (int)std::floor((d.z_loc_max - z) / d.dz_elm);
    if (ex < 0 || ex >= nx || ey < 0 || ey >= ny || ez < 0 || ez >= nz) {
        why = "point rounds onto the outer edge of the domain";
        return -2;
    }
    const float sx = 2.0f * ((x - d.x_loc_min) / d.dx_elm - (float)ex) - 1.0f;
    const float sy = 2.0f * ((y - d.y_loc_min) / d.dy_elm - (float)ey) - 1.0f;
    const float sz = 2.0f * ((d.z_loc_max - z) / d.dz_elm - (float)ez) - 1.0f;
    std::vector<float> pts = gll_points<float>(lpd);
    std::vector<float> lx = lagrange_basis(sx, pts), ly = lagrange_basis(sy, pts), lz = lagrange_basis(sz, pts);
    const int P = lpd + 1;
    for (int k = 0; k < P; ++k)
        for (int j = 0; j < P; ++j)
            for (int i = 0; i < P; ++i) vanderm[i + P * (j + P * k)] = lx[i] * ly[j] * lz[k];
    elem[0] = ex;
    elem[1] = ey;
    elem[2] = ez;
    return 0;
}

// Built-in source-time functions, src/misc/source_signature_mod.f90:50-147,
// sampled at t = i*dt (src/config/source.f90:583-586).
int source_signature(int wavelet, float onset, float width, float dt, int nt, float *out) {
    const float pi = pi_val<float>();
    for (int i = 0; i < nt; ++i) {
        const float t = (float)i * dt;
        float s = 0.0f;
        if (wavelet == 0) {  // DELTA
            s = (t == onset) ? 1.0f : 0.0f;
        } else if (wavelet == 1) {  // RICKER: 2*(0.5 + a*(t-T)^2)*exp(a*(t-T)^2), a = -(pi/width)^2
            const float pw = pi / width;
            const float a = -(pw * pw);
            const float d2 = (t - onset) * (t - onset);
            s = 2.0f * (0.5f + a * d2) * std::exp(a * d2);
        } else if (wavelet == 2) {  // GAUSS
            const float q = (t - onset) / width;
            s = std::exp(-(q * q));
        } else if (wavelet == 3) {  // SIN**3 on (onset, onset+width)
            if (onset < t && t < onset + width) {
                const float v = std::sin(pi * (t - onset) / width);
                s = v * v * v;
            }
        } else if (wavelet == 4) {  // BRUNE
            if (t >= onset) s = (t - onset) / (width * width) * std::exp(-(t - onset) / width);
        } else {
            return -1;
        }
        out[i] = s;
    }
    return 0;
}

// Algorithmic bytes of one step: element-local sigma R+W (48), lambda+mu (8),
// A,B,C (12, anisotropic only), memory variables R+W (48 per mechanism) and
// tau (4, visco-elastic only); per unique point v R+W (24) and 1/M (4). Only
// sigma, memory and v scale with the batch. Scaled by elem_bytes/4 for FP64.
long long algorithmic_bytes(long long nloc, long long nuni, int n_sls, bool aniso, int S, int elem_bytes) {
    const long long per_sim_loc = 48 + 48LL * n_sls;
    const long long shared_loc = 8 + (aniso ? 12 : 0) + (n_sls > 0 ? 4 : 0);
    const long long per_sim_uni = 24, shared_uni = 4;
    long long b = nloc * (per_sim_loc * S + shared_loc) + nuni * (per_sim_uni * S + shared_uni);
    return b * elem_bytes / 4;
}

template std::vector<float> gll_points<float>(int);
template std::vector<double> gll_points<double>(int);
template std::vector<float> gll_quadrature_weights<float>(int);
template std::vector<double> gll_quadrature_weights<double>(int);
template std::vector<float> lagrange_derivative_matrix<float>(int);
template std::vector<double> lagrange_derivative_matrix<double>(int);
template Domain<float> make_domain<float>(int, int, int, float, float, float, float, float, float);
template Domain<double> make_domain<double>(int, int, int, float, float, float, float, float, float);
template std::vector<float> element_coordinates<float>(int, int, float, float);
template std::vector<double> element_coordinates<double>(int, int, double, double);
template void taper_profiles<float>(int, int, int, int, int, float, const Domain<float> &, std::vector<float> &,
                                    std::vector<float> &, std::vector<float> &);
template void taper_profiles<double>(int, int, int, int, int, double, const Domain<double> &, std::vector<double> &,
                                     std::vector<double> &, std::vector<double> &);

}  // namespace sesnt
