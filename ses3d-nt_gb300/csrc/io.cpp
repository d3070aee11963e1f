// File formats around the time step: the raw model/field files the reference
// reads and writes (native float32, Fortran order (nx,ny,nz,P,P,P), no
// header; src/mpi_parallel_io.F90:121-341) and SAC traces
// (src/sac_io/sac_io_mod.f90:163-222,453-506), plus the Courant number and
// maximum-frequency report of src/model_paras.F90:464-561.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/sesnt.h"
#include "sesnt_internal.h"

namespace {

thread_local std::string g_io_error;

int io_fail(int code, const std::string &msg) {
    g_io_error = msg;
    return code;
}

bool file_exists(const char *path) {
    struct stat st;
    return stat(path, &st) == 0;
}

// Day of the year (1..366) of a Gregorian date (src/sac_io/sac_header_mod.f90,
// iday: iday(2012,1,1) = 1, iday(2012,10,11) = 285).
int day_of_year(int y, int m, int d) {
    static const int cum[12] = {0, 31, 59, 90, 120, 151, 181, 212, 243, 273, 304, 334};
    if (m < 1 || m > 12) return -12345;
    const bool leap = (y % 4 == 0 && y % 100 != 0) || (y % 400 == 0);
    return cum[m - 1] + d + ((leap && m > 2) ? 1 : 0);
}

// SAC header words (0-based): 70 floats, 35 ints, 5 logicals (4-byte), then
// 48 four-character words (KSTNM, KEVNM (16 chars), KHOLE, ..., KCMPNM,
// KNETWK, KDATRD, KINST).
enum SacWord {
    DELTA = 0, SCALE = 3, B = 5, E = 6, STLA = 31, STLO = 32, STDP = 34,
    NZYEAR = 70, NZJDAY = 71, NZHOUR = 72, NZMIN = 73, NZSEC = 74, NZMSEC = 75, NVHDR = 76, NPTS = 79,
    IFTYPE = 85, ISYNTH = 94,
    LEVEN = 105, LPSPOL = 106, LOVROK = 107, LCALDA = 108,
    KSTNM = 110, KEVNM = 112, KHOLE = 116, KCMPNM = 150, KNETWK = 152,
};

void put_chars(unsigned char *hdr, int word, const char *s, int len) {
    char buf[16];
    const size_t n = s ? strnlen(s, len) : 0;
    for (int i = 0; i < len; ++i) buf[i] = i < (int)n ? s[i] : ' ';  // blank padded like a Fortran assignment
    std::memcpy(hdr + 4 * word, buf, len);
}

std::string trimmed(const char *s, int len) {
    std::string t(s ? s : "", s ? strnlen(s, len) : 0);
    while (!t.empty() && t.back() == ' ') t.pop_back();
    return t;
}

}  // namespace

extern "C" {

const char *sesnt_io_last_error(void) { return g_io_error.c_str(); }

// Reference raw layout reader with the size check of
// src/mpi_parallel_io.F90:300-309 ("wrong file size").
int sesnt_read_raw_field(const char *path, int nx, int ny, int nz, int lpd, float *out) {
    if (!path || !out || nx < 1 || ny < 1 || nz < 1 || lpd < 1) return io_fail(SESNT_EINVAL, "invalid arguments");
    const long long P = lpd + 1, n = (long long)nx * ny * nz * P * P * P;
    FILE *f = std::fopen(path, "rb");
    if (!f) return io_fail(SESNT_EINVAL, std::string("cannot open model file '") + path + "': " + std::strerror(errno));
    std::fseek(f, 0, SEEK_END);
    const long long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (size != n * (long long)sizeof(float)) {
        std::fclose(f);
        char b[512];
        std::snprintf(b, sizeof b, "could not read '%s': wrong file size (%lld bytes, expected %lld for %dx%dx%dx%lldx%lldx%lld float32)",
                      path, size, n * 4, nx, ny, nz, P, P, P);
        return io_fail(SESNT_EINVAL, b);
    }
    const size_t got = std::fread(out, sizeof(float), (size_t)n, f);
    std::fclose(f);
    if ((long long)got != n) return io_fail(SESNT_EINVAL, std::string("short read from '") + path + "'");
    return SESNT_OK;
}

// Raw layout writer (src/mpi_parallel_io.F90:121-190): refuses to replace an
// existing file unless override is set (MPI_MODE_EXCL otherwise).
int sesnt_write_raw_field(const char *path, int nx, int ny, int nz, int lpd, const float *data, int override) {
    if (!path || !data || nx < 1 || ny < 1 || nz < 1 || lpd < 1) return io_fail(SESNT_EINVAL, "invalid arguments");
    if (!override && file_exists(path))
        return io_fail(SESNT_EINVAL, std::string("'") + path + "' exists and override is off");
    const long long P = lpd + 1, n = (long long)nx * ny * nz * P * P * P;
    FILE *f = std::fopen(path, "wb");
    if (!f) return io_fail(SESNT_EINVAL, std::string("cannot create '") + path + "': " + std::strerror(errno));
    const size_t put = std::fwrite(data, sizeof(float), (size_t)n, f);
    const int rc = std::fclose(f);
    if ((long long)put != n || rc != 0) return io_fail(SESNT_EINVAL, std::string("write to '") + path + "' failed");
    return SESNT_OK;
}

// SAC trace of one receiver channel, laid out as construct_trace sets it
// (src/sac_io/sac_io_mod.f90:178-222) on the reference's header defaults
// (:45-48): undefined floats and ints -12345, NVHDR 6, LEVEN true, the other
// logicals false, undefined strings "-12345..".
int sesnt_write_sac(const char *path, const sesnt_sac_info_t *info, const float *data, int npts) {
    if (!path || !info || !data || npts < 1) return io_fail(SESNT_EINVAL, "invalid arguments");
    if (!info->override && file_exists(path))
        return io_fail(SESNT_EINVAL, std::string("'") + path + "' exists and override is off");
    unsigned char hdr[158 * 4];
    float fl[70];
    int in[35];
    for (float &x : fl) x = -12345.0f;
    for (int &x : in) x = -12345;
    in[NVHDR - 70] = 6;
    std::memcpy(hdr, fl, sizeof fl);
    std::memcpy(hdr + 280, in, sizeof in);
    const int lg[5] = {1, 0, 0, 0, 0};
    std::memcpy(hdr + 420, lg, sizeof lg);
    for (int w = 110; w < 158; w += 2) std::memcpy(hdr + 4 * w, "-12345..", 8);
    auto setf = [&](int w, float v) { std::memcpy(hdr + 4 * w, &v, 4); };
    auto seti = [&](int w, int v) { std::memcpy(hdr + 4 * w, &v, 4); };
    setf(STLA, info->lat);
    setf(STLO, info->lon);
    setf(STDP, info->depth);
    put_chars(hdr, KEVNM, info->event, 16);
    put_chars(hdr, KNETWK, info->network, 8);
    put_chars(hdr, KSTNM, info->station, 8);
    put_chars(hdr, KHOLE, info->location, 8);
    put_chars(hdr, KCMPNM, info->channel, 8);
    seti(LOVROK, info->override ? 1 : 0);
    const int *dtm = info->date_time;
    seti(NZYEAR, dtm[0]);
    seti(NZJDAY, day_of_year(dtm[0], dtm[1], dtm[2]));
    seti(NZHOUR, dtm[4]);
    seti(NZMIN, dtm[5]);
    seti(NZSEC, dtm[6]);
    seti(NZMSEC, dtm[7]);
    setf(DELTA, info->dt);
    seti(NPTS, npts);
    setf(B, 0.0f);
    setf(E, info->dt * (float)npts);
    seti(IFTYPE, 1);
    seti(ISYNTH, 2);
    setf(SCALE, 1.0f);
    FILE *f = std::fopen(path, "wb");
    if (!f) return io_fail(SESNT_EINVAL, std::string("cannot create '") + path + "': " + std::strerror(errno));
    size_t ok = std::fwrite(hdr, 1, sizeof hdr, f) == sizeof hdr;
    ok = ok && std::fwrite(data, sizeof(float), (size_t)npts, f) == (size_t)npts;
    const int rc = std::fclose(f);
    if (!ok || rc != 0) return io_fail(SESNT_EINVAL, std::string("write to '") + path + "' failed");
    return SESNT_OK;
}

// "[network].[station].[location].[channel].sac" with trailing blanks
// removed (auto_file_name, src/sac_io/sac_io_mod.f90:407-427).
int sesnt_sac_file_name(const sesnt_sac_info_t *info, char *out, int out_len) {
    if (!info || !out || out_len < 1) return SESNT_EINVAL;
    const std::string s = trimmed(info->network, 8) + "." + trimmed(info->station, 8) + "." +
                          trimmed(info->location, 8) + "." + trimmed(info->channel, 8) + ".sac";
    if ((int)s.size() + 1 > out_len) return SESNT_ERANGE;
    std::memcpy(out, s.c_str(), s.size() + 1);
    return SESNT_OK;
}

int sesnt_day_of_year(int year, int month, int day) { return day_of_year(year, month, day); }

// Courant number and maximum resolved frequency of a model on a grid,
// src/model_paras.F90:464-494 (f_c_loc, two elements per minimal wavelength)
// and :529-561 (cfl_loc), in float32 with the reference's operation order.
// Model arrays in the reference raw layout; out[0] = Courant number,
// out[1] = f_c [Hz].
int sesnt_courant(const sesnt_grid_t *g, const float *rhoinv, const float *lambda, const float *mu, float out[2]) {
    using sesnt::Domain;
    if (!g || !rhoinv || !lambda || !mu || !out || g->lpd < sesnt::kMinLpd || g->lpd > sesnt::kMaxLpd)
        return io_fail(SESNT_EINVAL, "invalid arguments");
    const int N = g->lpd, P = N + 1;
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const long long nel = (long long)nx * ny * nz;
    Domain<float> d = sesnt::make_domain<float>(nx, ny, nz, g->lat_min, g->lat_max, g->lon_min, g->lon_max,
                                                g->rad_min, g->rad_max);
    std::vector<float> th = sesnt::element_coordinates<float>(nx, N, d.x_loc_min, d.x_loc_max);
    std::vector<float> ph = sesnt::element_coordinates<float>(ny, N, d.y_loc_min, d.y_loc_max);
    std::vector<float> rr = sesnt::element_coordinates<float>(nz, N, d.z_loc_max, d.z_loc_min);
    float cfl[3] = {-INFINITY, -INFINITY, -INFINITY}, fc[3] = {INFINITY, INFINITY, INFINITY};
    const float dt = g->dt, s = 2.0f;
    auto at = [&](int ex, int ey, int ez, int i, int j, int k) -> long long {
        return ex + (long long)nx * (ey + (long long)ny * ez) + nel * (i + (long long)P * (j + (long long)P * k));
    };
    auto speeds = [&](long long a, float &cp, float &cs) {
        cp = std::sqrt((lambda[a] + 2.0f * mu[a]) * rhoinv[a]);
        cs = std::sqrt(mu[a] * rhoinv[a]);
    };
    for (int ez = 0; ez < nz; ++ez)
        for (int ey = 0; ey < ny; ++ey)
            for (int ex = 0; ex < nx; ++ex)
                for (int k = 0; k < P; ++k)
                    for (int j = 0; j < P; ++j) {
                        const float r = rr[ez * P + k];
                        float sum_i = 0.0f;
                        for (int i = 0; i < P; ++i) {
                            float cp, cs;
                            speeds(at(ex, ey, ez, i, j, k), cp, cs);
                            const float vmax = cs < cp ? cp : cs, vmin = cs > cp ? cp : cs;
                            sum_i = sum_i + vmin;
                            const float sin_t = std::sin(th[ex * P + i]);
                            if (i >= 1) cfl[0] = std::fmax(cfl[0], vmax / (r * (th[ex * P + i] - th[ex * P + i - 1])));
                            if (j >= 1)
                                cfl[1] = std::fmax(cfl[1], vmax / (r * sin_t * (ph[ey * P + j] - ph[ey * P + j - 1])));
                            if (k >= 1) cfl[2] = std::fmax(cfl[2], vmax / (rr[ez * P + k - 1] - r));
                        }
                        const float vmean = sum_i / (float)P;
                        if (vmean > 0.0f) fc[0] = std::fmin(fc[0], vmean / s / (r * d.dx_elm));
                    }
    // phi and r directions of f_c: mean over j at i = 0 radius*sin, mean over k
    for (int ez = 0; ez < nz; ++ez)
        for (int ey = 0; ey < ny; ++ey)
            for (int ex = 0; ex < nx; ++ex)
                for (int k = 0; k < P; ++k)
                    for (int i = 0; i < P; ++i) {
                        float sum_j = 0.0f;
                        for (int j = 0; j < P; ++j) {
                            float cp, cs;
                            speeds(at(ex, ey, ez, i, j, k), cp, cs);
                            sum_j = sum_j + (cs > cp ? cp : cs);
                        }
                        const float vmean = sum_j / (float)P;
                        const float arc = rr[ez * P + k] * std::sin(th[ex * P + i]) * d.dy_elm;
                        if (vmean > 0.0f) fc[1] = std::fmin(fc[1], vmean / s / arc);
                    }
    for (int ez = 0; ez < nz; ++ez)
        for (int ey = 0; ey < ny; ++ey)
            for (int ex = 0; ex < nx; ++ex)
                for (int j = 0; j < P; ++j)
                    for (int i = 0; i < P; ++i) {
                        float sum_k = 0.0f;
                        for (int k = 0; k < P; ++k) {
                            float cp, cs;
                            speeds(at(ex, ey, ez, i, j, k), cp, cs);
                            sum_k = sum_k + (cs > cp ? cp : cs);
                        }
                        const float vmean = sum_k / (float)P;
                        if (vmean > 0.0f) fc[2] = std::fmin(fc[2], vmean / s / d.dz_elm);
                    }
    out[0] = std::fmax(cfl[0] * dt, std::fmax(cfl[1] * dt, cfl[2] * dt));
    out[1] = std::fmin(fc[0], std::fmin(fc[1], fc[2]));
    return SESNT_OK;
}

}  // extern "C"
