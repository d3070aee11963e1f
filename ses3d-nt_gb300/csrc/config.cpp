// Reader of the reference's configuration file: Fortran NAMELIST groups
// &grid &model &time &general &source_mt &source_sf &receiver &output_* ...
// (src/parser/parser.f90:45-137, CONFIG_FILE_FORMAT.md), and the forward
// workflow of the reference driver built on it (src/ses3d-nt.F90:77-275):
// read the config and the raw model files, locate sources and receivers,
// run every step on the GPU, write one SAC trace per receiver channel.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/sesnt.h"
#include "sesnt_internal.h"

namespace {

thread_local std::string g_cfg_error;

struct Value {
    enum Kind { STR, INT, REAL, BOOL } kind;
    std::string text;  // string content, or the literal
};

struct Group {
    std::string name;
    std::vector<std::pair<std::string, std::vector<Value>>> items;  // in file order
    const std::vector<Value> *find(const std::string &key) const {
        for (auto &kv : items)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

std::string lower(std::string s) {
    for (char &c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

bool is_number(const std::string &t, bool &integer) {
    if (t.empty()) return false;
    std::string u = t;
    for (char &c : u)
        if (c == 'd' || c == 'D') c = 'e';
    char *end = nullptr;
    std::strtod(u.c_str(), &end);
    if (!end || *end != '\0') return false;
    integer = u.find_first_of(".eE") == std::string::npos;
    return true;
}

Value classify(const std::string &tok) {
    const std::string l = lower(tok);
    if (l == "t" || l == ".true." || l == ".t.") return {Value::BOOL, "T"};
    if (l == "f" || l == ".false." || l == ".f.") return {Value::BOOL, "F"};
    bool integer = false;
    if (is_number(tok, integer)) return {integer ? Value::INT : Value::REAL, tok};
    return {Value::STR, tok};
}

// Tokenise one group body: names, '=', values (quoted strings keep their
// content), with '!' comments and ',' separators removed.
struct Tok {
    std::string s;
    bool quoted, eq;
};

bool parse(const std::string &text, std::vector<Group> &out, std::string &err) {
    size_t i = 0, n = text.size();
    Group *cur = nullptr;
    std::vector<Tok> toks;
    auto flush = [&]() -> bool {
        // key = v v v key = v ...
        std::string key;
        for (size_t a = 0; a < toks.size(); ++a) {
            if (a + 1 < toks.size() && toks[a + 1].eq && !toks[a].quoted) {
                key = lower(toks[a].s);
                const size_t paren = key.find('(');
                if (paren != std::string::npos) key = key.substr(0, paren);
                cur->items.push_back({key, {}});
                ++a;  // skip '='
                continue;
            }
            if (toks[a].eq || key.empty()) {
                err = "invalid assignment in group &" + cur->name;
                return false;
            }
            Value v = toks[a].quoted ? Value{Value::STR, toks[a].s} : classify(toks[a].s);
            // repeat counts r*value
            const size_t star = toks[a].quoted ? std::string::npos : toks[a].s.find('*');
            if (star != std::string::npos && star > 0) {
                const int r = std::atoi(toks[a].s.substr(0, star).c_str());
                Value w = classify(toks[a].s.substr(star + 1));
                for (int q = 0; q < r; ++q) cur->items.back().second.push_back(w);
                continue;
            }
            cur->items.back().second.push_back(v);
        }
        toks.clear();
        return true;
    };
    while (i < n) {
        const char c = text[i];
        if (c == '!') {
            while (i < n && text[i] != '\n') ++i;
            continue;
        }
        if (!cur) {
            if (c == '&' || c == '$') {
                size_t j = i + 1;
                while (j < n && (std::isalnum((unsigned char)text[j]) || text[j] == '_')) ++j;
                const std::string name = lower(text.substr(i + 1, j - i - 1));
                if (name == "end") {
                    i = j;
                    continue;
                }
                out.push_back({name, {}});
                cur = &out.back();
                i = j;
                continue;
            }
            ++i;
            continue;
        }
        if (std::isspace((unsigned char)c) || c == ',') {
            ++i;
            continue;
        }
        if (c == '/' || c == '&' || c == '$') {
            if (!flush()) return false;
            cur = nullptr;
            if (c == '&' || c == '$') {  // "&end" terminator
                size_t j = i + 1;
                while (j < n && std::isalpha((unsigned char)text[j])) ++j;
                i = j;
            } else {
                ++i;
            }
            continue;
        }
        if (c == '=') {
            toks.push_back({"=", false, true});
            ++i;
            continue;
        }
        if (c == '\'' || c == '"') {
            std::string s;
            size_t j = i + 1;
            while (j < n) {
                if (text[j] == c) {
                    if (j + 1 < n && text[j + 1] == c) {  // doubled quote
                        s += c;
                        j += 2;
                        continue;
                    }
                    break;
                }
                s += text[j++];
            }
            if (j >= n) {
                err = "unterminated string";
                return false;
            }
            toks.push_back({s, true, false});
            i = j + 1;
            continue;
        }
        size_t j = i;
        while (j < n && !std::isspace((unsigned char)text[j]) && text[j] != ',' && text[j] != '=' && text[j] != '/' &&
               text[j] != '!' && text[j] != '\'' && text[j] != '"')
            ++j;
        // a '(' ... ')' subscript stays glued to the name
        toks.push_back({text.substr(i, j - i), false, false});
        i = j;
    }
    if (cur) {
        err = "group &" + cur->name + " not terminated by '/'";
        return false;
    }
    return true;
}

std::string json_escape(const std::string &s) {
    std::string o;
    for (char c : s) {
        if (c == '"' || c == '\\') o += '\\';
        if ((unsigned char)c < 0x20) {
            char b[8];
            std::snprintf(b, sizeof b, "\\u%04x", c);
            o += b;
            continue;
        }
        o += c;
    }
    return o;
}

std::string json_value(const Value &v) {
    switch (v.kind) {
        case Value::STR: return "\"" + json_escape(v.text) + "\"";
        case Value::BOOL: return v.text == "T" ? "true" : "false";
        case Value::INT: return std::to_string(std::atoll(v.text.c_str()));
        case Value::REAL: {
            std::string u = v.text;
            for (char &c : u)
                if (c == 'd' || c == 'D') c = 'e';
            char b[64];
            std::snprintf(b, sizeof b, "%.17g", std::strtod(u.c_str(), nullptr));
            std::string s = b;
            if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
            return s;
        }
    }
    return "null";
}

}  // namespace

struct sesnt_config {
    std::vector<Group> groups;
    const Group *first(const char *name) const {
        for (auto &g : groups)
            if (g.name == name) return &g;
        return nullptr;
    }
};

namespace {

const Group *nth(const sesnt_config *c, const char *name, int idx) {
    int k = 0;
    for (auto &g : c->groups)
        if (g.name == name && k++ == idx) return &g;
    return nullptr;
}

bool get_num(const Group *g, const char *key, double &out) {
    if (!g) return false;
    const std::vector<Value> *v = g->find(key);
    if (!v || v->empty() || (v->front().kind != Value::INT && v->front().kind != Value::REAL)) return false;
    std::string u = v->front().text;
    for (char &ch : u)
        if (ch == 'd' || ch == 'D') ch = 'e';
    out = std::strtod(u.c_str(), nullptr);
    return true;
}

bool get_nums(const Group *g, const char *key, std::vector<float> &out) {
    out.clear();
    if (!g) return false;
    const std::vector<Value> *v = g->find(key);
    if (!v) return false;
    for (auto &x : *v) {
        if (x.kind != Value::INT && x.kind != Value::REAL) return false;
        std::string u = x.text;
        for (char &ch : u)
            if (ch == 'd' || ch == 'D') ch = 'e';
        out.push_back((float)std::strtod(u.c_str(), nullptr));
    }
    return true;
}

std::string get_str(const Group *g, const char *key, const char *dflt) {
    if (!g) return dflt;
    const std::vector<Value> *v = g->find(key);
    if (!v || v->empty()) return dflt;
    return v->front().text;
}

// Fixed-width text field, truncated or zero filled (no terminator needed).
void put_field(char *dst, const std::string &src, size_t len) {
    std::memset(dst, 0, len);
    std::memcpy(dst, src.data(), std::min(len, src.size()));
}

bool get_bool(const Group *g, const char *key, bool dflt) {
    if (!g) return dflt;
    const std::vector<Value> *v = g->find(key);
    if (!v || v->empty() || v->front().kind != Value::BOOL) return dflt;
    return v->front().text == "T";
}

}  // namespace

extern "C" {

const char *sesnt_config_last_error(void) { return g_cfg_error.c_str(); }

int sesnt_config_load(const char *path, sesnt_config_t **out) {
    if (!path || !out) return SESNT_EINVAL;
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        g_cfg_error = std::string("cannot open config file '") + path + "'";
        return SESNT_EINVAL;
    }
    std::string text;
    char buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
    std::fclose(f);
    std::unique_ptr<sesnt_config> c(new sesnt_config());
    std::string err;
    if (!parse(text, c->groups, err)) {
        g_cfg_error = std::string(path) + ": " + err;
        return SESNT_EINVAL;
    }
    *out = c.release();
    return SESNT_OK;
}

int sesnt_config_free(sesnt_config_t *c) {
    delete c;
    return SESNT_OK;
}

int sesnt_config_count(const sesnt_config_t *c, const char *group) {
    if (!c || !group) return SESNT_EINVAL;
    int k = 0;
    const std::string g = lower(group);
    for (auto &x : c->groups)
        if (x.name == g) ++k;
    return k;
}

// JSON image of the parsed file: {"group": [{key: value or [values]}, ...]},
// groups in first-appearance order (the shape of ses3dpy's namelist2dict).
int sesnt_config_json(const sesnt_config_t *c, char *out, long long out_len, long long *needed) {
    if (!c) return SESNT_EINVAL;
    std::vector<std::string> names;
    for (auto &g : c->groups)
        if (std::find(names.begin(), names.end(), g.name) == names.end()) names.push_back(g.name);
    std::ostringstream o;
    o << "{";
    for (size_t a = 0; a < names.size(); ++a) {
        o << (a ? ", " : "") << "\"" << names[a] << "\": [";
        bool firstg = true;
        for (auto &g : c->groups) {
            if (g.name != names[a]) continue;
            o << (firstg ? "" : ", ") << "{";
            firstg = false;
            for (size_t b = 0; b < g.items.size(); ++b) {
                o << (b ? ", " : "") << "\"" << json_escape(g.items[b].first) << "\": ";
                const auto &vals = g.items[b].second;
                if (vals.size() == 1) {
                    o << json_value(vals[0]);
                } else {
                    o << "[";
                    for (size_t q = 0; q < vals.size(); ++q) o << (q ? ", " : "") << json_value(vals[q]);
                    o << "]";
                }
            }
            o << "}";
        }
        o << "]";
    }
    o << "}";
    const std::string s = o.str();
    if (needed) *needed = (long long)s.size() + 1;
    if (!out) return SESNT_OK;
    if ((long long)s.size() + 1 > out_len) return SESNT_ERANGE;
    std::memcpy(out, s.c_str(), s.size() + 1);
    return SESNT_OK;
}

// &grid, &model, &time into the grid struct (src/config/config.F90:97-233
// checks apply at sesnt_create). n_sls is 3 when the model names a q file.
int sesnt_config_grid(const sesnt_config_t *c, sesnt_grid_t *g) {
    if (!c || !g) return SESNT_EINVAL;
    const Group *gr = c->first("grid"), *md = c->first("model"), *tm = c->first("time");
    if (!gr || !md || !tm) {
        g_cfg_error = "config needs &grid, &model and &time groups";
        return SESNT_EINVAL;
    }
    double v;
    std::memset(g, 0, sizeof *g);
    auto need = [&](const Group *grp, const char *key, double &dst) -> bool {
        if (!get_num(grp, key, dst)) {
            g_cfg_error = std::string("missing or non-numeric '") + key + "' in &" + grp->name;
            return false;
        }
        return true;
    };
    int *ik[4] = {&g->nx, &g->ny, &g->nz, &g->lpd};
    const char *in[4] = {"nx", "ny", "nz", "lpd"};
    for (int q = 0; q < 4; ++q) {
        if (!need(gr, in[q], v)) return SESNT_EINVAL;
        *ik[q] = (int)v;
    }
    g->taper_width = get_num(gr, "taper_width", v) ? (int)v : 0;
    g->taper_slope = get_num(gr, "taper_slope", v) ? (float)v : 1.0f;
    const char *mk[6] = {"lat_min", "lat_max", "lon_min", "lon_max", "rad_min", "rad_max"};
    float *mv[6] = {&g->lat_min, &g->lat_max, &g->lon_min, &g->lon_max, &g->rad_min, &g->rad_max};
    for (int q = 0; q < 6; ++q) {
        if (!need(md, mk[q], v)) return SESNT_EINVAL;
        *mv[q] = (float)v;
    }
    if (!need(tm, "dt", v)) return SESNT_EINVAL;
    g->dt = (float)v;
    if (!need(tm, "nt", v)) return SESNT_EINVAL;
    g->nt = (int)v;
    const std::string q = get_str(md, "q", "N/A");
    g->n_sls = (q != "N/A" && !q.empty()) ? sesnt::kNsls : 0;
    g->precision = 4;
    g->batch = 1;
    g->flags = 0;
    return SESNT_OK;
}

// Value of `key` in the idx-th `group` as text (strings unquoted, logicals
// T/F, several values separated by single blanks).
int sesnt_config_get(const sesnt_config_t *c, const char *group, int idx, const char *key, char *out, int out_len) {
    if (!c || !group || !key || !out || out_len < 1) return SESNT_EINVAL;
    const Group *g = nth(c, lower(group).c_str(), idx);
    if (!g) return SESNT_ENOTFOUND;
    const std::vector<Value> *v = g->find(lower(key));
    if (!v) return SESNT_ENOTFOUND;
    std::string s;
    for (size_t q = 0; q < v->size(); ++q) s += (q ? " " : "") + (*v)[q].text;
    if ((int)s.size() + 1 > out_len) return SESNT_ERANGE;
    std::memcpy(out, s.c_str(), s.size() + 1);
    return SESNT_OK;
}

// The reference's forward workflow on the GPU. Model files are read relative
// to the working directory, as the reference opens them. Points outside the
// domain are skipped with a warning (src/config/point.f90:208-218); receiver
// channels other than vx, vy, vz are skipped with a warning. One SAC file per
// receiver channel is written to prefix + "[net].[sta].[loc].[cha].sac".
int sesnt_forward(const char *config_path, int precision, int *n_traces) {
    if (n_traces) *n_traces = 0;
    sesnt_config_t *cfg = nullptr;
    int rc = sesnt_config_load(config_path, &cfg);
    if (rc) return rc;
    std::unique_ptr<sesnt_config, int (*)(sesnt_config_t *)> guard(cfg, sesnt_config_free);
    sesnt_grid_t g;
    if ((rc = sesnt_config_grid(cfg, &g))) return rc;
    g.precision = precision == 8 ? 8 : 4;
    const Group *md = cfg->first("model");
    const double model_type_v = [&] { double v = -1; get_num(md, "model_type", v); return v; }();
    if (model_type_v != -1.0 && cfg->first("model")->find("model_type")) {
        g_cfg_error = "only file models (model_type = -1) are supported on the GPU path";
        return SESNT_EUNSUPPORTED;
    }
    const long long P = g.lpd + 1, n = (long long)g.nx * g.ny * g.nz * P * P * P;
    std::vector<float> arr[7];
    const char *keys[7] = {"rhoinv", "lambda", "mu", "a", "b", "c", "q"};
    for (int q = 0; q < 7; ++q) {
        const std::string fn = get_str(md, keys[q], "N/A");
        if (fn == "N/A" || fn.empty()) {
            if (q < 3) {
                g_cfg_error = std::string("'") + keys[q] + "' model-file must be given";
                return SESNT_EINVAL;
            }
            continue;
        }
        arr[q].resize(n);
        if ((rc = sesnt_read_raw_field(fn.c_str(), g.nx, g.ny, g.nz, g.lpd, arr[q].data()))) {
            g_cfg_error = sesnt_io_last_error();
            return rc;
        }
    }
    // &output_raw groups (src/output_raw.f90:175-253): one snapshot series per
    // attribute, with the defaults of volume_snapshot_cls' constructor
    // (src/volume_snapshot.f90:71-113)
    struct Raw { std::string attr, prefix; int start, inc, end; bool override; };
    std::vector<Raw> raws;
    for (int q = 0;; ++q) {
        const Group *og = nth(cfg, "output_raw", q);
        if (!og) break;
        double start = 1, inc = -1, end = -1;
        get_num(og, "timestep_start", start);
        get_num(og, "timestep_increment", inc);
        get_num(og, "timestep_end", end);
        const std::string prefix = get_str(og, "prefix", "./");
        const bool over = get_bool(og, "override", false);
        if (const std::vector<Value> *at = og->find("attributes"))
            for (auto &a : *at) {
                std::string l = lower(a.text);
                while (!l.empty() && l.back() == ' ') l.pop_back();
                if (l.empty()) continue;
                raws.push_back({l, prefix, (int)start, (int)inc, end < 0 ? g.nt : (int)end, over});
                const int id = sesnt_field_id(l.c_str());
                if (id >= SESNT_FIELD_EXX && id <= SESNT_FIELD_EZZ) g.flags |= SESNT_FLAG_STRAIN;
            }
    }
    sesnt_t *h = nullptr;
    if ((rc = sesnt_create(&g, &h))) {
        g_cfg_error = sesnt_last_error(nullptr);
        return rc;
    }
    std::unique_ptr<sesnt_t, int (*)(sesnt_t *)> hguard(h, sesnt_destroy);
    auto ptr = [&](int q) -> const float * { return arr[q].empty() ? nullptr : arr[q].data(); };
    if ((rc = sesnt_set_model(h, ptr(0), ptr(1), ptr(2), ptr(3), ptr(4), ptr(5), ptr(6)))) {
        g_cfg_error = sesnt_last_error(h);
        return rc;
    }
    for (const Raw &r : raws) {
        // wavefield and device-held fields: snapshots written behind the steps
        const int id = sesnt_field_id(r.attr.c_str());
        const bool host = r.attr == "rho" || r.attr == "vs" || r.attr == "cs" || r.attr == "vp" || r.attr == "cp" ||
                          r.attr == "q";
        if (id >= 0 && id != SESNT_FIELD_MASS && !host) {
            if ((rc = sesnt_add_snapshot(h, 0, id, r.start, r.inc, r.end, r.prefix.c_str(), r.attr.c_str(),
                                         r.override ? 1 : 0)) < 0) {
                g_cfg_error = sesnt_last_error(h);
                return rc;
            }
            continue;
        }
        if (!host) {
            std::fprintf(stderr, "warning: snapshot attribute '%s' not available on the GPU path; skipped\n",
                         r.attr.c_str());
            continue;
        }
        if (r.start < 1 || r.inc < 1 || r.inc > g.nt || r.end < r.start) {
            g_cfg_error = "timestep range of &output_raw out of range";
            return SESNT_ERANGE;
        }
        // static model fields (get_field, src/volume_snapshot.f90:259-285):
        // rho = 1/rhoinv where rhoinv > 0 (src/model_paras.F90:399-403)
        std::vector<float> f(n);
        for (long long i = 0; i < n; ++i) {
            const float ri = arr[0][i], rho = ri > 0.0f ? 1.0f / ri : 0.0f;
            if (r.attr == "rho") f[i] = rho;
            else if (r.attr == "vs" || r.attr == "cs") f[i] = std::sqrt(arr[2][i] / rho);
            else if (r.attr == "vp" || r.attr == "cp") f[i] = std::sqrt((arr[1][i] + 2.0f * arr[2][i]) / rho);
            else f[i] = arr[6].empty() ? std::numeric_limits<float>::max() : arr[6][i];
        }
        for (int it = r.start; it <= std::min(r.end, g.nt); it += r.inc) {
            const std::string path = r.prefix + r.attr + "_" + std::to_string(it) + ".vol";
            if ((rc = sesnt_write_raw_field(path.c_str(), g.nx, g.ny, g.nz, g.lpd, f.data(), r.override ? 1 : 0))) {
                g_cfg_error = sesnt_io_last_error();
                return rc;
            }
        }
    }
    const Group *tm = cfg->first("time");
    std::vector<float> vm(P * P * P), stf(g.nt), comp;
    int elem[3];
    for (const char *kind : {"source_mt", "source_sf"}) {
        for (int s = 0;; ++s) {
            const Group *sg = nth(cfg, kind, s);
            if (!sg) break;
            double lat = 0, lon = 0, depth = 0, onset = 0, width = 0;
            get_num(sg, "lat", lat); get_num(sg, "lon", lon); get_num(sg, "depth", depth);
            get_num(sg, "onset", onset); get_num(sg, "width", width);
            if (sesnt_locate_point(&g, (float)lat, (float)lon, (float)depth, elem, vm.data())) {
                std::fprintf(stderr, "warning: source (%g, %g, %g) not in the computational domain; skipped\n", lat,
                             lon, depth);
                continue;
            }
            const std::string wl = get_str(sg, "wavelet", "RICKER");
            const char *names[5] = {"DELTA", "RICKER", "GAUSS", "SIN**3", "BRUNE"};
            int code = -1;
            for (int q = 0; q < 5; ++q)
                if (wl == names[q]) code = q;
            if (code < 0) {
                g_cfg_error = "source wavelet '" + wl + "' (file wavelets are not supported)";
                return SESNT_EUNSUPPORTED;
            }
            sesnt_source_signature(code, (float)onset, (float)width, g.dt, g.nt, stf.data());
            const bool mt = std::strcmp(kind, "source_mt") == 0;
            if (!get_nums(sg, mt ? "moment_tensor" : "direction", comp) || comp.size() != (mt ? 6u : 3u)) {
                g_cfg_error = std::string("invalid ") + (mt ? "moment_tensor" : "direction") + " in &" + kind;
                return SESNT_EINVAL;
            }
            if ((rc = sesnt_add_source(h, 0, elem[0], elem[1], elem[2], vm.data(), mt ? SESNT_SOURCE_MT : SESNT_SOURCE_SF,
                                       comp.data(), stf.data(), g.nt))) {
                g_cfg_error = sesnt_last_error(h);
                return rc;
            }
        }
    }
    struct Rec {
        const Group *grp;
        int index;
        std::vector<std::pair<std::string, unsigned>> chans;  // attribute, channel bit
        double lat, lon, depth;
    };
    std::vector<Rec> recs;
    for (int r = 0;; ++r) {
        const Group *rg = nth(cfg, "receiver", r);
        if (!rg) break;
        double lat = 0, lon = 0, depth = 0;
        get_num(rg, "lat", lat); get_num(rg, "lon", lon); get_num(rg, "depth", depth);
        // receiver attributes (construct_channel_container_receiver,
        // src/config/channel_mod.f90:270-342); unknown ones are dropped with
        // a warning (src/config/receiver.f90:389-398)
        static const std::pair<const char *, unsigned> kAttr[] = {
            {"vx", SESNT_CH_VX}, {"n", SESNT_CH_N}, {"vy", SESNT_CH_VY}, {"e", SESNT_CH_VY}, {"vz", SESNT_CH_VZ},
            {"z", SESNT_CH_VZ}, {"rot_vx", SESNT_CH_ROT_VX}, {"rot_vy", SESNT_CH_ROT_VY},
            {"rot_vz", SESNT_CH_ROT_VZ}, {"mxx", SESNT_CH_MXX}, {"mxy", SESNT_CH_MXY}, {"myx", SESNT_CH_MXY},
            {"mxz", SESNT_CH_MXZ}, {"mzx", SESNT_CH_MXZ}, {"myy", SESNT_CH_MYY}, {"myz", SESNT_CH_MYZ},
            {"mzy", SESNT_CH_MYZ}, {"mzz", SESNT_CH_MZZ}, {"fx", SESNT_CH_FX}, {"fy", SESNT_CH_FY},
            {"fz", SESNT_CH_FZ}};
        unsigned mask = 0;
        std::vector<std::pair<std::string, unsigned>> chans;
        if (const std::vector<Value> *at = rg->find("attributes"))
            for (auto &a : *at) {
                std::string l = lower(a.text);
                while (!l.empty() && l.back() == ' ') l.pop_back();
                unsigned bit = 0;
                for (auto &k : kAttr)
                    if (l == k.first) bit = k.second;
                if (!bit) {
                    std::fprintf(stderr, "warning: unknown receiver attribute '%s' dropped\n", a.text.c_str());
                    continue;
                }
                mask |= bit;
                chans.push_back({l, bit});
            }
        if (!mask) continue;
        if (sesnt_locate_point(&g, (float)lat, (float)lon, (float)depth, elem, vm.data())) {
            std::fprintf(stderr, "warning: receiver (%g, %g, %g) not in the computational domain; skipped\n", lat, lon,
                         depth);
            continue;
        }
        const int idx = sesnt_add_receiver(h, elem[0], elem[1], elem[2], vm.data(), mask);
        if (idx < 0) {
            g_cfg_error = sesnt_last_error(h);
            return idx;
        }
        recs.push_back({rg, idx, chans, lat, lon, depth});
    }
    if ((rc = sesnt_run(h, 1, g.nt))) {
        g_cfg_error = sesnt_last_error(h);
        return rc;
    }
    if ((rc = sesnt_snapshots_wait(h))) {
        g_cfg_error = sesnt_last_error(h);
        return rc;
    }
    std::vector<float> trace(g.nt);
    // date_time from &time, else now (src/config/config.F90:218-225)
    int dtm[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
    std::vector<float> dv;
    if (get_nums(tm, "date_time", dv) && dv.size() == 8)
        for (int q = 0; q < 8; ++q) dtm[q] = (int)dv[q];
    if (dtm[0] == -1) {
        std::time_t t = std::time(nullptr);
        std::tm u = *std::gmtime(&t);
        const int now[8] = {u.tm_year + 1900, u.tm_mon + 1, u.tm_mday, 0, u.tm_hour, u.tm_min, u.tm_sec, 0};
        std::memcpy(dtm, now, sizeof now);
    }
    const std::string event = get_str(cfg->first("general"), "event_name", "ses3d-nt event");
    int written = 0;
    for (const Rec &r : recs)
        for (const auto &ch : r.chans) {
            if ((rc = sesnt_get_trace(h, 0, r.index, ch.second, trace.data()))) {
                g_cfg_error = sesnt_last_error(h);
                return rc;
            }
            sesnt_sac_info_t info;
            std::memset(&info, 0, sizeof info);
            info.lat = (float)r.lat;
            info.lon = (float)r.lon;
            info.depth = (float)r.depth;
            info.dt = g.dt;
            put_field(info.network, get_str(r.grp, "network", "Ses3d-NT"), 8);  // default: parser.f90:438
            put_field(info.station, get_str(r.grp, "station", ""), 8);
            put_field(info.location, get_str(r.grp, "location", ""), 8);
            put_field(info.channel, ch.first, 8);
            put_field(info.event, event, 16);
            info.override = get_bool(r.grp, "override", false) ? 1 : 0;
            std::memcpy(info.date_time, dtm, sizeof dtm);
            char name[256];
            sesnt_sac_file_name(&info, name, sizeof name);
            const std::string path = get_str(r.grp, "prefix", "./") + name;
            if ((rc = sesnt_write_sac(path.c_str(), &info, trace.data(), g.nt))) {
                g_cfg_error = sesnt_io_last_error();
                return rc;
            }
            ++written;
        }
    if (n_traces) *n_traces = written;
    return SESNT_OK;
}

}  // extern "C"
