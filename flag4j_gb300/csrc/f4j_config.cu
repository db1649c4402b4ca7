// f4j_config.cu -- the dense-product dispatcher's configuration files (host code).
//
// Flag4j reads three java.util.Properties files from ./configs at class
// initialisation, falling back to built-in defaults when a file is absent:
//   ReDeMatMult.properties   ReDeMatMultDispatchConfigs
//     (src/main/java/org/flag4j/linalg/ops/dispatch/configs/ReDeMatMultDispatchConfigs.java:52-121)
//   CmDeMatMult.properties   Cm128DeMatMultDispatchConfigs (same directory, :52-108)
//   GeneralConfigs.properties Configurations (src/main/java/org/flag4j/concurrency/Configurations.java:65-88)
// This file reads the same files with the same keys, defaults and number
// syntax (Integer.parseInt, Double.parseDouble), plus one key of its own,
// gpuGemmMode = auto | split | plain | exact, which picks the GPU path of
// F4J_MODE_AUTO above the reference's small-product threshold.  It also
// restates the dispatchers' kernel choice (ReDeMatMultDispatcher.getFunc,
// ReDeMatMultDispatcher.java:184-237; Cm128DeMatMultDispatcher.getFunc,
// Cm128DeMatMultDispatcher.java:184-226) so a caller can see which CPU kernel
// the reference would have run for a shape.
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>

#include "f4j_internal.cuh"

namespace {

struct Configs {
    f4j_dispatch_config dc[2];  // [0] real (ReDeMatMult), [1] complex (CmDeMatMult)
    int32_t block_size;
    int32_t parallelism;        // resolved thread count (ThreadManager.setParallelismLevel)
    int32_t general_loaded;
};

std::mutex g_cfg_mu;
bool g_cfg_init = false;
Configs g_cfg;

void defaults(Configs* c) {
    // ReDeMatMultDispatchConfigs.java:52-87
    f4j_dispatch_config& r = c->dc[0];
    r = f4j_dispatch_config{};
    r.cache_size = 64;
    r.aspect_threshold = 2.0;
    r.small_threshold = 2450;
    r.square_mt_standard_threshold = 50;
    r.square_mt_reordered_threshold = 2048;
    r.wide_mt_reordered_threshold = 25;
    r.square_sequential_vec_threshold = 256;
    r.min_dim_small_threshold = 10;
    r.gpu_gemm_mode = F4J_MODE_AUTO;
    // Cm128DeMatMultDispatchConfigs.java:52-83 (no vector threshold: complex
    // matrix-vector products always take MT_STRD_VEC_AS_MAT)
    f4j_dispatch_config& z = c->dc[1];
    z = f4j_dispatch_config{};
    z.cache_size = 64;
    z.aspect_threshold = 2.0;
    z.small_threshold = 512;
    z.square_mt_standard_threshold = 60;
    z.square_mt_reordered_threshold = 2048;
    z.wide_mt_reordered_threshold = 25;
    z.square_sequential_vec_threshold = 0;
    z.min_dim_small_threshold = 10;
    z.gpu_gemm_mode = F4J_MODE_AUTO;
    // Configurations.java:60-65: blockSize 64, parallelism = available processors
    c->block_size = 64;
    unsigned hw = std::thread::hardware_concurrency();
    c->parallelism = hw ? (int32_t)hw : 1;
    c->general_loaded = 0;
}

// ---- java.util.Properties.load, the parts a .properties file can contain
// Natural lines joined by a trailing odd run of backslashes; blank lines and
// lines whose first non-blank character is '#' or '!' skipped; the key ends at
// the first unescaped '=', ':' or blank; blanks, then one '=' or ':', then
// blanks separate it from the value; escapes \t \n \r \f \uXXXX and \c -> c.
// Trailing blanks stay in the value (Properties keeps them).
std::string unescape(const std::string& s) {
    std::string out;
    for (size_t i = 0; i < s.size(); i++) {
        char ch = s[i];
        if (ch != '\\' || i + 1 >= s.size()) {
            out += ch;
            continue;
        }
        char e = s[++i];
        if (e == 't') out += '\t';
        else if (e == 'n') out += '\n';
        else if (e == 'r') out += '\r';
        else if (e == 'f') out += '\f';
        else if (e == 'u' && i + 4 < s.size() && isxdigit((unsigned char)s[i + 1]) &&
                 isxdigit((unsigned char)s[i + 2]) && isxdigit((unsigned char)s[i + 3]) &&
                 isxdigit((unsigned char)s[i + 4])) {
            const unsigned v = (unsigned)strtoul(s.substr(i + 1, 4).c_str(), nullptr, 16);
            i += 4;
            if (v < 0x80) {
                out += (char)v;
            } else if (v < 0x800) {
                out += (char)(0xC0 | (v >> 6));
                out += (char)(0x80 | (v & 63));
            } else {
                out += (char)(0xE0 | (v >> 12));
                out += (char)(0x80 | ((v >> 6) & 63));
                out += (char)(0x80 | (v & 63));
            }
        } else {
            out += e;
        }
    }
    return out;
}

bool is_blank(char c) { return c == ' ' || c == '\t' || c == '\f'; }

// Returns false when the file cannot be opened (the reference then keeps its defaults).
bool load_properties(const std::string& path, std::map<std::string, std::string>* props) {
    std::ifstream in(path, std::ios::binary);
    if (!in) return false;
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string text = ss.str();
    std::string logical;
    bool cont = false;
    size_t pos = 0;
    while (pos <= text.size()) {
        size_t eol = text.find_first_of("\r\n", pos);
        std::string line = text.substr(pos, eol == std::string::npos ? std::string::npos : eol - pos);
        if (eol == std::string::npos) pos = text.size() + 1;
        else pos = (text[eol] == '\r' && eol + 1 < text.size() && text[eol + 1] == '\n') ? eol + 2 : eol + 1;
        size_t b = 0;
        while (b < line.size() && is_blank(line[b])) b++;
        if (!cont) {
            if (b == line.size()) continue;                  // blank line
            if (line[b] == '#' || line[b] == '!') continue;  // comment line
        }
        line = line.substr(b);
        size_t nbs = 0;
        while (nbs < line.size() && line[line.size() - 1 - nbs] == '\\') nbs++;
        const bool next_cont = (nbs % 2) == 1;
        if (next_cont) line.pop_back();
        logical += line;
        cont = next_cont;
        if (cont && pos <= text.size()) continue;
        // split key / value
        size_t i = 0;
        std::string key;
        for (; i < logical.size(); i++) {
            char c = logical[i];
            if (c == '\\' && i + 1 < logical.size()) {
                key += c;
                key += logical[++i];
                continue;
            }
            if (c == '=' || c == ':' || is_blank(c)) break;
            key += c;
        }
        while (i < logical.size() && is_blank(logical[i])) i++;
        if (i < logical.size() && (logical[i] == '=' || logical[i] == ':')) i++;
        while (i < logical.size() && is_blank(logical[i])) i++;
        (*props)[unescape(key)] = unescape(logical.substr(i));
        logical.clear();
        cont = false;
    }
    return true;
}

// Integer.parseInt: optional sign, decimal digits only, within int32.
bool java_parse_int(const std::string& s, int32_t* out) {
    size_t i = 0;
    bool neg = false;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) neg = s[i++] == '-';
    if (i >= s.size()) return false;
    long long v = 0;
    for (; i < s.size(); i++) {
        if (s[i] < '0' || s[i] > '9') return false;
        v = v * 10 + (s[i] - '0');
        if (v > (long long)INT_MAX + 1) return false;
    }
    if (neg) v = -v;
    if (v > INT_MAX || v < INT_MIN) return false;
    *out = (int32_t)v;
    return true;
}

// Double.parseDouble for decimal text: surrounding blanks trimmed, an optional
// d / D / f / F suffix, "Infinity" and "NaN" spelled as Java spells them.
bool java_parse_double(const std::string& raw, double* out) {
    size_t a = 0, b = raw.size();
    while (a < b && (unsigned char)raw[a] <= ' ') a++;
    while (b > a && (unsigned char)raw[b - 1] <= ' ') b--;
    std::string s = raw.substr(a, b - a);
    if (s.empty()) return false;
    std::string body = s;
    size_t sgn = (body[0] == '+' || body[0] == '-') ? 1 : 0;
    if (body.compare(sgn, std::string::npos, "Infinity") == 0) {
        *out = body[0] == '-' ? -INFINITY : INFINITY;
        return true;
    }
    if (body.compare(sgn, std::string::npos, "NaN") == 0) {
        *out = NAN;
        return true;
    }
    char last = body.back();
    if (last == 'd' || last == 'D' || last == 'f' || last == 'F') body.pop_back();
    // decimal digits with an optional point and exponent only (no hex, no inf/nan words here)
    bool digit = false;
    for (size_t i = sgn; i < body.size(); i++) {
        const char c = body[i];
        if (c >= '0' && c <= '9') digit = true;
        else if (c == '.' || c == 'e' || c == 'E' || ((c == '+' || c == '-') && (body[i - 1] == 'e' || body[i - 1] == 'E')))
            continue;
        else return false;
    }
    if (!digit) return false;
    char* end = nullptr;
    errno = 0;
    double v = strtod(body.c_str(), &end);
    if (end != body.c_str() + body.size()) return false;
    *out = v;
    return true;
}

int parse_error(const std::string& path, const char* key, const std::string& value) {
    return f4j_fail(F4J_ERR_ARG, "%s: %s: NumberFormatException: For input string: \"%s\"", path.c_str(), key,
                    value.c_str());
}

int apply_dispatch(const std::string& path, const std::map<std::string, std::string>& p, bool real,
                   f4j_dispatch_config* d) {
    auto it = p.end();
    if ((it = p.find("cacheSize")) != p.end() && !java_parse_double(it->second, &d->cache_size))
        return parse_error(path, "cacheSize", it->second);
    if ((it = p.find("aspectThreshold")) != p.end() && !java_parse_double(it->second, &d->aspect_threshold))
        return parse_error(path, "aspectThreshold", it->second);
    struct { const char* key; int32_t* dst; } ints[] = {
        {"smallThreshold", &d->small_threshold},
        {"squareMtStandardThreshold", &d->square_mt_standard_threshold},
        {"squareMtReorderedThreshold", &d->square_mt_reordered_threshold},
        {"wideMtReorderedThreshold", &d->wide_mt_reordered_threshold},
        // the reference reads this key for real products only; its shipped file
        // spells it squareStandardVecThreshold, which no code reads
        {real ? "squareSequentialVecThreshold" : nullptr, &d->square_sequential_vec_threshold},
        {"minDimSmallThreshold", &d->min_dim_small_threshold},
    };
    for (auto& e : ints) {
        if (!e.key) continue;
        if ((it = p.find(e.key)) != p.end() && !java_parse_int(it->second, e.dst))
            return parse_error(path, e.key, it->second);
    }
    return F4J_OK;
}

int parse_mode(const std::string& path, const std::string& raw, int32_t* mode) {
    std::string s;
    for (char c : raw)
        if (!is_blank(c)) s += (char)tolower((unsigned char)c);
    if (s == "auto") *mode = F4J_MODE_AUTO;
    else if (s == "split") *mode = F4J_MODE_SPLIT;
    else if (s == "plain") *mode = F4J_MODE_PLAIN;
    else if (s == "exact") *mode = F4J_MODE_EXACT;
    else return f4j_fail(F4J_ERR_ARG, "%s: gpuGemmMode must be auto, split, plain or exact, got \"%s\"", path.c_str(),
                         raw.c_str());
    return F4J_OK;
}

int load_dir(const char* dir, Configs* c) {
    defaults(c);
    const std::string base = std::string(dir ? dir : "./configs") + "/";
    int32_t general_mode = F4J_MODE_AUTO;
    bool general_mode_set = false;
    {
        std::map<std::string, std::string> p;
        const std::string path = base + "GeneralConfigs.properties";
        if (load_properties(path, &p)) {
            c->general_loaded = 1;
            auto it = p.end();
            int32_t v = 0;
            if ((it = p.find("blockSize")) != p.end()) {
                if (!java_parse_int(it->second, &v)) return parse_error(path, "blockSize", it->second);
                c->block_size = v;
            }
            if ((it = p.find("parallelism")) != p.end()) {
                if (!java_parse_int(it->second, &v)) return parse_error(path, "parallelism", it->second);
                if (v <= 0) v = c->parallelism + v;  // ThreadManager.setParallelismLevel
                c->parallelism = v < 1 ? 1 : v;
            }
            if ((it = p.find("gpuGemmMode")) != p.end()) {
                int rc = parse_mode(path, it->second, &general_mode);
                if (rc) return rc;
                general_mode_set = true;
            }
        }
    }
    const char* names[2] = {"ReDeMatMult.properties", "CmDeMatMult.properties"};
    for (int t = 0; t < 2; t++) {
        std::map<std::string, std::string> p;
        const std::string path = base + names[t];
        f4j_dispatch_config* d = &c->dc[t];
        if (general_mode_set) d->gpu_gemm_mode = general_mode;
        if (!load_properties(path, &p)) continue;
        d->loaded = 1;
        int rc = apply_dispatch(path, p, t == 0, d);
        if (rc) return rc;
        auto it = p.find("gpuGemmMode");
        if (it != p.end()) {
            rc = parse_mode(path, it->second, &d->gpu_gemm_mode);
            if (rc) return rc;
        }
    }
    return F4J_OK;
}

const Configs& current() {
    // first use: ./configs relative to the working directory, as the
    // reference's static initialisers do (a malformed file leaves the defaults)
    if (!g_cfg_init) {
        Configs c;
        if (load_dir(nullptr, &c) != F4J_OK) defaults(&c);
        g_cfg = c;
        g_cfg_init = true;
    }
    return g_cfg;
}

const char* kKernelNames[] = {"STRD", "REORD", "BLK", "BLK_REORD", "MT_STRD", "MT_REORD", "MT_BLK", "MT_BLK_REORD",
                              "STRD_VEC_AS_MAT", "BLK_VEC_AS_MAT", "MT_STRD_VEC_AS_MAT", "MT_BLK_VEC_AS_MAT"};

// The kernel the reference's dispatcher runs for A (m x k) times B (k x n).
int ref_kernel(const f4j_dispatch_config& d, bool cplx, int64_t m, int64_t n, int64_t k) {
    if (m * k + k * n < (int64_t)d.small_threshold) return F4J_REF_STRD;  // dispatch()'s small path
    // getFunc names: aShape (m, n_ref = k), bShape (k, k_ref = n)
    const int64_t M = m, Nr = k, Kr = n;
    if (Kr == 1) {
        if (cplx) return F4J_REF_MT_STRD_VEC_AS_MAT;
        const double ar = (double)(M > Nr ? M : Nr) / (double)(M < Nr ? M : Nr);
        if (ar <= 4 * d.aspect_threshold) return M < d.square_sequential_vec_threshold ? F4J_REF_BLK_VEC_AS_MAT
                                                                                     : F4J_REF_MT_BLK_VEC_AS_MAT;
        return F4J_REF_BLK_VEC_AS_MAT;
    }
    const int64_t mn = Kr < (M < Nr ? M : Nr) ? Kr : (M < Nr ? M : Nr);
    const int64_t mx = Kr > (M > Nr ? M : Nr) ? Kr : (M > Nr ? M : Nr);
    const double ar = (double)mx / (double)mn;
    if (ar <= d.aspect_threshold) {
        if (Nr < d.square_mt_standard_threshold) return F4J_REF_MT_STRD;
        if (Nr < d.square_mt_reordered_threshold) return F4J_REF_MT_REORD;
        return F4J_REF_MT_BLK_REORD;
    }
    if (M == mx) return mn < d.min_dim_small_threshold ? F4J_REF_STRD : F4J_REF_MT_REORD;
    if (Nr == mx) {
        if (mn < d.min_dim_small_threshold) return F4J_REF_STRD;
        return M < d.wide_mt_reordered_threshold ? F4J_REF_MT_STRD : F4J_REF_MT_REORD;
    }
    return mn < d.min_dim_small_threshold ? F4J_REF_REORD : F4J_REF_MT_REORD;
}

}  // namespace

int f4j_resolve_mode(bool cplx, int64_t m, int64_t n, int64_t k, int mode) {
    if (mode != F4J_MODE_AUTO) return mode;
    f4j_dispatch_config d;
    {
        std::lock_guard<std::mutex> lk(g_cfg_mu);
        d = current().dc[cplx ? 1 : 0];
    }
    // the reference's small-product rule (ReDeMatMultDispatcher.java:159-168,
    // Cm128DeMatMultDispatcher.java:156-167): its standard kernel, i.e. EXACT
    if (m * k + k * n < (int64_t)d.small_threshold) return F4J_MODE_EXACT;
    // products of a few microseconds of work keep the reference's order too
    const double work = (cplx ? 8.0 : 2.0) * (double)m * (double)n * (double)k;
    if (work <= (double)(1 << 24)) return F4J_MODE_EXACT;
    return d.gpu_gemm_mode == F4J_MODE_AUTO ? F4J_MODE_SPLIT : d.gpu_gemm_mode;
}

extern "C" int f4j_config_load(const char* dir) {
    Configs c;
    int rc = load_dir(dir, &c);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    g_cfg = c;
    g_cfg_init = true;
    return F4J_OK;
}

extern "C" int f4j_config_reset(void) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    defaults(&g_cfg);
    g_cfg_init = true;
    return F4J_OK;
}

extern "C" int f4j_config_get(int cplx, f4j_dispatch_config* out) {
    if (!out) return f4j_fail(F4J_ERR_ARG, "null output pointer");
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    *out = current().dc[cplx ? 1 : 0];
    return F4J_OK;
}

extern "C" int f4j_config_general(int32_t* block_size, int32_t* parallelism) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    const Configs& c = current();
    if (block_size) *block_size = c.block_size;
    if (parallelism) *parallelism = c.parallelism;
    return F4J_OK;
}

extern "C" int f4j_dispatch(int cplx, int64_t m, int64_t n, int64_t k, int mode, int32_t* mode_out,
                            int32_t* ref_kernel_out) {
    if (m < 0 || n < 0 || k < 0) return f4j_fail(F4J_ERR_ARG, "negative dimension");
    if (mode < F4J_MODE_PLAIN || mode > F4J_MODE_EXACT) return f4j_fail(F4J_ERR_ARG, "bad mode %d", mode);
    f4j_dispatch_config d;
    {
        std::lock_guard<std::mutex> lk(g_cfg_mu);
        d = current().dc[cplx ? 1 : 0];
    }
    if (mode_out) *mode_out = f4j_resolve_mode(cplx != 0, m, n, k, mode);
    if (ref_kernel_out) *ref_kernel_out = (m == 0 || n == 0 || k == 0) ? F4J_REF_STRD : ref_kernel(d, cplx != 0, m, n, k);
    return F4J_OK;
}

extern "C" const char* f4j_ref_kernel_name(int code) {
    if (code < 0 || code >= (int)(sizeof kKernelNames / sizeof kKernelNames[0])) return "?";
    return kKernelNames[code];
}
