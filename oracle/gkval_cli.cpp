/*
 * gkval_cli.cpp -- `gkval`, the GEOKERR validation harness (TEST INFRASTRUCTURE).
 *
 * Compares the library's GPU GEOKERR path with the CPU restatement of
 * GEOKERR (geokerr_oracle.cpp) sample by sample, the way the reference's
 * gkval compares its CUDA port with the Fortran GEOKERR
 * (geokerr_port/validation/gkval_cli.c, gkval_validator.c:227-407):
 *
 *   gkval init --run-id ID [--grid adaptive_lambda|uniform_lambda|uniform_affine]
 *              [--size S] [--delta D] [--atol A] [--rtol R] [--max-ulps N]
 *              [--quant-lsb Q] [--profile bitexact|default|relaxed]
 *              [--hash sha256|placeholder] [--runs-dir DIR]
 *   gkval validate ID [--cases FILE] [--port gpu|oracle] [--lib PATH]
 *              [--resume] [--plant FIELD:INDEX:ULPS] [--runs-dir DIR]
 *   gkval audit ID [--runs-dir DIR]
 *   gkval diff ID CASE [FIELD] [--runs-dir DIR]
 *
 * Run layout (validation/README.md:38-46): <runs-dir>/<ID>/manifest.json,
 * ledger.ndjson (one line per case), cursor.json, fail_windows/<case>/.
 *
 * Reference solver: the CPU restatement of geokerr_eval_lambda.  Port
 * solvers: "gpu" calls the library's geokerr_complete_stream_cuda through
 * its C ABI (the call the reference's CUDA adapter makes,
 * gkval_adapters.c:666-695); "oracle" runs the restatement against itself
 * (a pipeline self-check).  --plant moves one port sample of one field by a
 * number of ULPs after the port solver returns, so tests can check that a
 * planted difference is found where it was put.  Like the reference's CUDA
 * adapter, the GPU port takes no t0, so cases with t0 != 0 differ in t by
 * t0 (a cases file normally leaves t0 at 0).
 *
 * Per case and field the S samples are compared in segments of 1024; phi is
 * unwrapped per segment; the first rejected sample ends the case and writes
 * a 32-sample fail window.  Passing segments are quantised and hashed into a
 * Merkle tree (field roots, then the case root).  Unlike the reference,
 * which writes no ledger line for a failing case, every case gets one
 * (success false, first failure, zero case root), each line also carries
 * the inputs (%.17g) and per-field maximum ULP and absolute differences,
 * and the cursor advances a whole case at a time, so a resumed run never
 * re-hashes a partial case.  `audit` recomputes every stored root from the
 * ledger's inputs and checks the fail windows' reference halves; `diff`
 * prints the samples of a case's fail windows.
 */
#include <algorithm>
#include <cerrno>
#include <cinttypes>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <dirent.h>
#include <dlfcn.h>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

extern "C" {
const char* gkv_field_name(int field);
int gkv_field_index(const char* s);
uint64_t gkv_ulp_distance(double a, double b);
int64_t gkv_first_fail(const double* a, const double* b, size_t n, double atol, double rtol, uint64_t max_ulps);
void gkv_unwrap(double* x, size_t n);
int gkv_quantize_block(const double* x, size_t n, int quant_lsb, uint64_t* q);
void gkv_hash_leaf(int hash_kind, const char* run_id, uint64_t case_id, int field, uint64_t start, uint64_t end,
                   const uint64_t* q, size_t n, uint8_t* out);
void gkv_merkle(int hash_kind, const uint8_t* hashes, size_t n, uint8_t* out);
int gkv_save_fail_window(const char* run_dir, uint64_t case_id, int field, uint64_t start, uint64_t end,
                         const double* ref, const double* port);
int gkv_load_fail_window(const char* run_dir, uint64_t case_id, int field, uint64_t start, uint64_t end,
                         double* ref, double* port);
void gkv_fail_window_bounds(uint64_t seg_start, uint64_t fail, uint64_t n, uint64_t width, uint64_t* start,
                            uint64_t* end);
int gkv_adaptive_grid(double u0, double mu0, double uf, double a, double lam, double q2, uint64_t S, double K,
                      double* lam0, double* dlam);
int gkv_check_fp_env(int fix);
void npo_geokerr_eval_lambda(double u0, double mu0, double uf, double a, double Lz, double Q2, double t0, double lam0,
                             double dlam, int S, double* u, double* mu, double* t, double* phi, double* affine,
                             int* tpmi, int* tpri, int* info);
}

namespace {

constexpr uint64_t kSeg = 1024;     // GKVAL_DEFAULT_SEG_SIZE
constexpr uint64_t kWindow = 32;    // GKVAL_DEFAULT_WINDOW_SIZE
constexpr int kFields = 5;

struct Manifest {
    std::string run_id, grid_type = "adaptive_lambda", hash = "sha256";
    uint64_t S = 4096;
    double delta = 1e-3, atol = 1e-12, rtol = 1e-12;
    uint64_t max_ulps = 2;
    int quant_lsb = 8;
    int hash_kind() const { return hash == "placeholder" ? 1 : 0; }
};

struct Inputs {
    double u0, mu0, uf, a, lam, q2, t0;
};

struct Trajectory {
    std::vector<double> f[kFields];
    int tpmi = -1, tpri = -1, info = 0;
};

std::string hex(const uint8_t* h) {
    static const char* d = "0123456789abcdef";
    std::string s;
    for (int i = 0; i < 32; ++i) { s += d[h[i] >> 4]; s += d[h[i] & 15]; }
    return s;
}

uint64_t bits_of(double x) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
}

double of_bits(uint64_t u) {
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

bool read_file(const std::string& p, std::string& out) {
    FILE* f = std::fopen(p.c_str(), "rb");
    if (!f) return false;
    char buf[4096];
    size_t k;
    out.clear();
    while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, k);
    std::fclose(f);
    return true;
}

bool write_atomic(const std::string& p, const std::string& s) {  // gkval_validator.c:42-60
    std::string tmp = p + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    bool ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
    ok = (std::fflush(f) == 0) && ok;
    ok = (fsync(fileno(f)) == 0) && ok;
    ok = (std::fclose(f) == 0) && ok;
    return ok && std::rename(tmp.c_str(), p.c_str()) == 0;
}

// Value text after "key": in a flat JSON object of our own format.
bool json_raw(const std::string& s, const char* key, std::string& v) {
    std::string k = std::string("\"") + key + "\"";
    size_t p = s.find(k);
    if (p == std::string::npos) return false;
    p = s.find(':', p + k.size());
    if (p == std::string::npos) return false;
    ++p;
    while (p < s.size() && (s[p] == ' ' || s[p] == '\t')) ++p;
    if (p < s.size() && s[p] == '"') {
        size_t q = s.find('"', p + 1);
        if (q == std::string::npos) return false;
        v = s.substr(p + 1, q - p - 1);
        return true;
    }
    size_t q = p;
    while (q < s.size() && s[q] != ',' && s[q] != '}' && s[q] != ']' && s[q] != '\n') ++q;
    v = s.substr(p, q - p);
    return true;
}

bool json_num(const std::string& s, const char* key, double& x) {
    std::string v;
    if (!json_raw(s, key, v)) return false;
    char* end = nullptr;
    x = std::strtod(v.c_str(), &end);
    return end != v.c_str();
}

bool json_u64(const std::string& s, const char* key, uint64_t& x) {
    std::string v;
    if (!json_raw(s, key, v)) return false;
    char* end = nullptr;
    x = std::strtoull(v.c_str(), &end, 10);
    return end != v.c_str();
}

std::string manifest_json(const Manifest& m) {  // gkval_validator.c:545-580, plus the hash in use
    char b[2048];
    std::snprintf(b, sizeof b,
                  "{\n  \"version\": \"1.0\",\n  \"run_id\": \"%s\",\n  \"geokerr_commit\": \"unknown\",\n"
                  "  \"port_commit\": \"unknown\",\n"
                  "  \"grid\": { \"type\": \"%s\", \"S\": %" PRIu64 ", \"delta\": %.15e },\n"
                  "  \"tolerances\": { \"atol\": %.15e, \"rtol\": %.15e, \"max_ulps\": %" PRIu64 " },\n"
                  "  \"quant_lsb\": %d,\n  \"hash\": \"%s\",\n"
                  "  \"fields\": [\"u\", \"mu\", \"t\", \"phi\", \"affine\"]\n}\n",
                  m.run_id.c_str(), m.grid_type.c_str(), m.S, m.delta, m.atol, m.rtol, m.max_ulps, m.quant_lsb,
                  m.hash.c_str());
    return b;
}

bool load_manifest(const std::string& dir, Manifest& m) {
    std::string s, v;
    if (!read_file(dir + "/manifest.json", s)) return false;
    double x;
    if (!json_raw(s, "run_id", m.run_id) || !json_raw(s, "type", m.grid_type)) return false;
    if (!json_u64(s, "S", m.S) || !json_num(s, "delta", m.delta) || !json_num(s, "atol", m.atol) ||
        !json_num(s, "rtol", m.rtol) || !json_u64(s, "max_ulps", m.max_ulps) || !json_num(s, "quant_lsb", x))
        return false;
    m.quant_lsb = (int)x;
    m.hash = json_raw(s, "hash", v) ? v : "placeholder";  // a reference manifest has no hash key
    return true;
}

// Grid of a case: lam0, dlam per the manifest's grid type.
bool case_grid(const Manifest& m, const Inputs& in, double& lam0, double& dlam) {
    if (m.grid_type == "adaptive_lambda") return gkv_adaptive_grid(in.u0, in.mu0, in.uf, in.a, in.lam, in.q2, m.S,
                                                                   6.0, &lam0, &dlam) == 0;
    lam0 = 0.0;
    dlam = m.delta;
    return true;
}

Trajectory run_reference(const Inputs& in, uint64_t S, double lam0, double dlam) {
    Trajectory t;
    for (auto& v : t.f) v.assign(S, 0.0);
    npo_geokerr_eval_lambda(in.u0, in.mu0, in.uf, in.a, in.lam, in.q2, in.t0, lam0, dlam, (int)S, t.f[0].data(),
                            t.f[1].data(), t.f[2].data(), t.f[3].data(), t.f[4].data(), &t.tpmi, &t.tpri, &t.info);
    return t;
}

typedef int (*stream_fn)(double, double, double, double, double, double, double, double, int, double*, double*,
                         double*, double*, double*);

std::string exe_dir() {
    char b[4096];
    ssize_t k = readlink("/proc/self/exe", b, sizeof b - 1);
    if (k <= 0) return ".";
    b[k] = 0;
    std::string p(b);
    return p.substr(0, p.rfind('/'));
}

struct Port {
    std::string kind = "gpu";
    stream_fn gpu = nullptr;
    int plant_field = -1;
    uint64_t plant_index = 0;
    int64_t plant_ulps = 0;

    bool open(const std::string& lib) {
        if (kind == "oracle") return true;
        std::string p = lib.empty() ? exe_dir() + "/../nullpath_gb300/lib/libnullpath_gb300.so" : lib;
        void* h = dlopen(p.c_str(), RTLD_NOW | RTLD_LOCAL);
        if (!h) {
            std::fprintf(stderr, "gkval: cannot load %s: %s\n", p.c_str(), dlerror());
            return false;
        }
        gpu = (stream_fn)dlsym(h, "geokerr_complete_stream_cuda");
        if (!gpu) std::fprintf(stderr, "gkval: geokerr_complete_stream_cuda not exported by %s\n", p.c_str());
        return gpu != nullptr;
    }

    // Returns 0 or the solver's error code; on error all samples are NaN
    // (gkval_adapters.c:684-692).
    int run(const Inputs& in, uint64_t S, double lam0, double dlam, Trajectory& t) {
        int rc = 0;
        if (kind == "oracle") {
            t = run_reference(in, S, lam0, dlam);
        } else {
            for (auto& v : t.f) v.assign(S, 0.0);
            rc = gpu(in.u0, in.uf, in.mu0, in.a, in.lam, in.q2, lam0, dlam, (int)S, t.f[0].data(), t.f[1].data(),
                     t.f[2].data(), t.f[3].data(), t.f[4].data());
            if (rc != 0)
                for (auto& v : t.f) v.assign(S, NAN);
        }
        if (plant_field >= 0 && plant_index < S) {
            double& x = t.f[plant_field][plant_index];
            int64_t bits = (int64_t)bits_of(x) + plant_ulps;
            x = of_bits((uint64_t)bits);
        }
        return rc;
    }
};

struct CaseResult {
    bool success = true;
    int fail_field = -1;
    uint64_t fail_index = 0;
    uint8_t field_roots[kFields][32] = {};
    uint8_t case_root[32] = {};
    uint64_t max_ulp[kFields] = {};
    double max_abs[kFields] = {};
    uint64_t nan_count = 0;
    double max_affine_drift = 0.0;
};

// Compares one case and, when write_windows, writes its fail window.
// Field roots and the case root hash the reference data of passing cases.
CaseResult compare_case(const Manifest& m, const std::string& run_dir, uint64_t case_id, Trajectory& ref,
                        Trajectory& port, bool write_windows) {
    CaseResult r;
    const uint64_t S = m.S;
    int hk = m.hash_kind();
    for (int f = 0; f < kFields; ++f) {
        std::vector<uint8_t> leaves;
        for (uint64_t s = 0; s < S; s += kSeg) {
            uint64_t n = std::min(kSeg, S - s);
            std::vector<double> a(ref.f[f].begin() + s, ref.f[f].begin() + s + n);
            std::vector<double> b(port.f[f].begin() + s, port.f[f].begin() + s + n);
            if (f == 3) { gkv_unwrap(a.data(), n); gkv_unwrap(b.data(), n); }
            for (uint64_t i = 0; i < n; ++i) {
                uint64_t u = gkv_ulp_distance(a[i], b[i]);
                r.max_ulp[f] = std::max(r.max_ulp[f], u);
                double d = std::fabs(a[i] - b[i]);
                if (d > r.max_abs[f] || std::isnan(d)) r.max_abs[f] = std::isnan(d) ? INFINITY : d;
                if (!std::isfinite(a[i]) || !std::isfinite(b[i])) r.nan_count++;
                if (f == 4) r.max_affine_drift = std::max(r.max_affine_drift, d);
            }
            if (!r.success) continue;  // first failure already recorded: statistics only
            int64_t ff = gkv_first_fail(a.data(), b.data(), n, m.atol, m.rtol, m.max_ulps);
            if (ff >= 0) {
                r.success = false;
                r.fail_field = f;
                r.fail_index = s + (uint64_t)ff;
                if (write_windows) {
                    uint64_t ws, we;
                    gkv_fail_window_bounds(s, (uint64_t)ff, n, kWindow, &ws, &we);
                    gkv_save_fail_window(run_dir.c_str(), case_id, f, ws, we, a.data() + (ws - s),
                                         b.data() + (ws - s));
                }
                continue;
            }
            std::vector<uint64_t> q(n);
            if (gkv_quantize_block(a.data(), n, m.quant_lsb, q.data()) != 0) {
                r.success = false;  // equal non-finite samples: no window, first_fail null
                continue;
            }
            uint8_t leaf[32];
            gkv_hash_leaf(hk, m.run_id.c_str(), case_id, f, s, s + n, q.data(), n, leaf);
            leaves.insert(leaves.end(), leaf, leaf + 32);
        }
        if (r.success) gkv_merkle(hk, leaves.data(), leaves.size() / 32, r.field_roots[f]);
    }
    // Invariants (gkval_validator.c:208-223): no NaN/Inf; affine drift within atol + rtol.
    if (r.nan_count > 0 || r.max_affine_drift > m.atol + m.rtol) r.success = false;
    if (r.success) gkv_merkle(hk, &r.field_roots[0][0], kFields, r.case_root);
    else std::memset(r.field_roots, 0, sizeof r.field_roots);
    return r;
}

std::string ledger_line(const Manifest& m, uint64_t case_id, const Inputs& in, double lam0, double dlam,
                        const Trajectory& ref, const CaseResult& r) {
    char b[4096];
    int k = std::snprintf(b, sizeof b,
                          "{\"run_id\":\"%s\",\"case_id\":%" PRIu64 ",\"success\":%s,"
                          "\"grid\":{\"S\":%" PRIu64 ",\"lam0_bits\":%" PRIu64 ",\"dlam_bits\":%" PRIu64 "},"
                          "\"tpmi\":%d,\"tpri\":%d,\"case_root\":\"%s\","
                          "\"inputs\":{\"u0\":%.17g,\"mu0\":%.17g,\"uf\":%.17g,\"a\":%.17g,\"lam\":%.17g,"
                          "\"q2\":%.17g,\"t0\":%.17g},",
                          m.run_id.c_str(), case_id, r.success ? "true" : "false", m.S, bits_of(lam0), bits_of(dlam),
                          ref.tpmi, ref.tpri, hex(r.case_root).c_str(), in.u0, in.mu0, in.uf, in.a, in.lam, in.q2,
                          in.t0);
    std::string s(b, k);
    if (r.fail_field >= 0) {
        std::snprintf(b, sizeof b, "\"first_fail\":{\"field\":\"%s\",\"index\":%" PRIu64 "},",
                      gkv_field_name(r.fail_field), r.fail_index);
        s += b;
    } else {
        s += "\"first_fail\":null,";
    }
    s += "\"max_ulp\":[";
    for (int f = 0; f < kFields; ++f) {
        std::snprintf(b, sizeof b, "%s%" PRIu64, f ? "," : "", r.max_ulp[f]);
        s += b;
    }
    s += "],\"max_abs\":[";
    for (int f = 0; f < kFields; ++f) {
        std::snprintf(b, sizeof b, "%s%.6e", f ? "," : "", std::isfinite(r.max_abs[f]) ? r.max_abs[f] : -1.0);
        s += b;
    }
    s += "]}";
    return s;
}

std::vector<Inputs> read_cases(const std::string& path, bool& ok) {
    ok = true;
    std::vector<Inputs> v;
    if (path.empty()) {  // the reference CLI's single built-in case (gkval_cli.c:177-180)
        v.push_back({0.1, 0.8, 0.01, 0.5, 2.0, 4.0, 0.0});
        return v;
    }
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) { ok = false; return v; }
    char line[1024];
    while (std::fgets(line, sizeof line, f)) {
        char* h = std::strchr(line, '#');
        if (h) *h = 0;
        Inputs in{};
        int k = std::sscanf(line, "%lf %lf %lf %lf %lf %lf %lf", &in.u0, &in.mu0, &in.uf, &in.a, &in.lam, &in.q2,
                            &in.t0);
        if (k <= 0) continue;
        if (k < 6) { ok = false; break; }
        if (k == 6) in.t0 = 0.0;
        v.push_back(in);
    }
    std::fclose(f);
    return v;
}

std::string opt(int argc, char** argv, const char* name, const char* dflt) {
    for (int i = 0; i + 1 < argc; ++i)
        if (std::strcmp(argv[i], name) == 0) return argv[i + 1];
    return dflt;
}

bool flag(int argc, char** argv, const char* name) {
    for (int i = 0; i < argc; ++i)
        if (std::strcmp(argv[i], name) == 0) return true;
    return false;
}

std::string run_dir_of(int argc, char** argv, const std::string& id) {
    return opt(argc, argv, "--runs-dir", "runs") + "/" + id;
}

int cmd_init(int argc, char** argv) {
    Manifest m;
    m.run_id = opt(argc, argv, "--run-id", "");
    if (m.run_id.empty()) {
        std::fprintf(stderr, "gkval init: --run-id is required\n");
        return 1;
    }
    m.grid_type = opt(argc, argv, "--grid", "adaptive_lambda");
    if (m.grid_type != "adaptive_lambda" && m.grid_type != "uniform_lambda" && m.grid_type != "uniform_affine") {
        std::fprintf(stderr, "gkval init: unknown grid %s\n", m.grid_type.c_str());
        return 1;
    }
    m.S = std::strtoull(opt(argc, argv, "--size", "4096").c_str(), nullptr, 10);
    m.delta = std::strtod(opt(argc, argv, "--delta", "1e-3").c_str(), nullptr);
    m.atol = std::strtod(opt(argc, argv, "--atol", "1e-12").c_str(), nullptr);
    m.rtol = std::strtod(opt(argc, argv, "--rtol", "1e-12").c_str(), nullptr);
    m.max_ulps = std::strtoull(opt(argc, argv, "--max-ulps", "2").c_str(), nullptr, 10);
    m.quant_lsb = std::atoi(opt(argc, argv, "--quant-lsb", "8").c_str());
    m.hash = opt(argc, argv, "--hash", "sha256");
    std::string prof = opt(argc, argv, "--profile", "");
    if (prof == "bitexact") {  // gkval_cli.c:57-62
        m.atol = m.rtol = 0.0;
        m.max_ulps = 0;
        m.quant_lsb = 0;
    } else if (prof == "relaxed") {  // the reference's relaxed runs' manifest
        m.atol = m.rtol = 1e-3;
        m.max_ulps = 100;
        m.quant_lsb = 8;
    } else if (!prof.empty() && prof != "default") {
        std::fprintf(stderr, "gkval init: unknown profile %s\n", prof.c_str());
        return 1;
    }
    if (m.S < 2 || m.quant_lsb < 0 || m.quant_lsb > 52 || (m.hash != "sha256" && m.hash != "placeholder")) {
        std::fprintf(stderr, "gkval init: invalid size, quant-lsb or hash\n");
        return 1;
    }
    std::string runs = opt(argc, argv, "--runs-dir", "runs"), dir = runs + "/" + m.run_id;
    if ((mkdir(runs.c_str(), 0755) != 0 && errno != EEXIST) || (mkdir(dir.c_str(), 0755) != 0 && errno != EEXIST) ||
        (mkdir((dir + "/fail_windows").c_str(), 0755) != 0 && errno != EEXIST)) {
        std::fprintf(stderr, "gkval init: cannot create %s\n", dir.c_str());
        return 1;
    }
    if (!write_atomic(dir + "/manifest.json", manifest_json(m)) ||
        !write_atomic(dir + "/cursor.json", "{\"case_id\": 0, \"field\": 0, \"start\": 0}\n")) {
        std::fprintf(stderr, "gkval init: cannot write the manifest\n");
        return 1;
    }
    std::printf("initialised %s (grid %s S=%" PRIu64 ", atol %.3g rtol %.3g max_ulps %" PRIu64 ", quant_lsb %d, %s)\n",
                dir.c_str(), m.grid_type.c_str(), m.S, m.atol, m.rtol, m.max_ulps, m.quant_lsb, m.hash.c_str());
    return 0;
}

int cmd_validate(int argc, char** argv) {
    if (argc < 1 || argv[0][0] == '-') {
        std::fprintf(stderr, "usage: gkval validate <run-id> [--cases FILE] [--port gpu|oracle] ...\n");
        return 1;
    }
    std::string dir = run_dir_of(argc, argv, argv[0]);
    Manifest m;
    if (!load_manifest(dir, m)) {
        std::fprintf(stderr, "gkval validate: cannot read %s/manifest.json\n", dir.c_str());
        return 1;
    }
    if (gkv_check_fp_env(1) != 0) std::fprintf(stderr, "gkval: warning: cannot set round-to-nearest\n");
    bool ok;
    std::vector<Inputs> cases = read_cases(opt(argc, argv, "--cases", ""), ok);
    if (!ok) {
        std::fprintf(stderr, "gkval validate: cannot read the cases file\n");
        return 1;
    }
    Port port;
    port.kind = opt(argc, argv, "--port", "gpu");
    if (port.kind != "gpu" && port.kind != "oracle") {
        std::fprintf(stderr, "gkval validate: unknown port %s\n", port.kind.c_str());
        return 1;
    }
    std::string plant = opt(argc, argv, "--plant", "");
    if (!plant.empty()) {
        char fname[32];
        unsigned long long idx;
        long long ulps;
        if (std::sscanf(plant.c_str(), "%31[^:]:%llu:%lld", fname, &idx, &ulps) != 3 ||
            gkv_field_index(fname) < 0) {
            std::fprintf(stderr, "gkval validate: --plant FIELD:INDEX:ULPS\n");
            return 1;
        }
        port.plant_field = gkv_field_index(fname);
        port.plant_index = idx;
        port.plant_ulps = ulps;
    }
    if (!port.open(opt(argc, argv, "--lib", ""))) return 1;

    uint64_t first = 0;
    if (flag(argc, argv, "--resume")) {
        std::string c;
        if (read_file(dir + "/cursor.json", c)) json_u64(c, "case_id", first);
    }
    uint64_t passed = 0, failed = 0;
    FILE* ledger = std::fopen((dir + "/ledger.ndjson").c_str(), "a");
    if (!ledger) {
        std::fprintf(stderr, "gkval validate: cannot open the ledger\n");
        return 1;
    }
    for (uint64_t id = first; id < cases.size(); ++id) {
        const Inputs& in = cases[id];
        double lam0, dlam;
        if (!case_grid(m, in, lam0, dlam)) {
            std::fprintf(stderr, "gkval validate: no grid for case %" PRIu64 "\n", id);
            std::fclose(ledger);
            return 1;
        }
        Trajectory ref = run_reference(in, m.S, lam0, dlam), pt;
        int rc = port.run(in, m.S, lam0, dlam, pt);
        if (rc != 0) std::fprintf(stderr, "gkval: port solver returned %d on case %" PRIu64 "\n", rc, id);
        CaseResult r = compare_case(m, dir, id, ref, pt, true);
        std::string line = ledger_line(m, id, in, lam0, dlam, ref, r);
        std::fprintf(ledger, "%s\n", line.c_str());
        std::fflush(ledger);
        fsync(fileno(ledger));
        char cur[128];
        std::snprintf(cur, sizeof cur, "{\"case_id\": %" PRIu64 ", \"field\": 0, \"start\": 0}\n", id + 1);
        write_atomic(dir + "/cursor.json", cur);
        (r.success ? passed : failed)++;
        std::printf("case %" PRIu64 ": %s", id, r.success ? "PASS" : "FAIL");
        if (r.fail_field >= 0)
            std::printf(" (first failure: %s[%" PRIu64 "])", gkv_field_name(r.fail_field), r.fail_index);
        std::printf("  max ulp u %" PRIu64 " mu %" PRIu64 " t %" PRIu64 " phi %" PRIu64 " affine %" PRIu64 "\n",
                    r.max_ulp[0], r.max_ulp[1], r.max_ulp[2], r.max_ulp[3], r.max_ulp[4]);
    }
    std::fclose(ledger);
    std::printf("%" PRIu64 " passed, %" PRIu64 " failed\n", passed, failed);
    return failed ? 2 : 0;
}

int cmd_audit(int argc, char** argv) {
    if (argc < 1 || argv[0][0] == '-') {
        std::fprintf(stderr, "usage: gkval audit <run-id>\n");
        return 1;
    }
    std::string dir = run_dir_of(argc, argv, argv[0]), led;
    Manifest m;
    if (!load_manifest(dir, m) || !read_file(dir + "/ledger.ndjson", led)) {
        std::fprintf(stderr, "gkval audit: cannot read %s\n", dir.c_str());
        return 1;
    }
    uint64_t lines = 0, bad = 0;
    size_t p = 0;
    while (p < led.size()) {
        size_t q = led.find('\n', p);
        if (q == std::string::npos) q = led.size();
        std::string L = led.substr(p, q - p);
        p = q + 1;
        if (L.empty()) continue;
        ++lines;
        uint64_t id = 0, lb = 0, db = 0;
        Inputs in{};
        std::string succ, root, run_id;
        bool parsed = json_u64(L, "case_id", id) && json_u64(L, "lam0_bits", lb) && json_u64(L, "dlam_bits", db) &&
                      json_raw(L, "success", succ) && json_raw(L, "case_root", root) &&
                      json_raw(L, "run_id", run_id) && json_num(L, "u0", in.u0) && json_num(L, "mu0", in.mu0) &&
                      json_num(L, "uf", in.uf) && json_num(L, "a", in.a) && json_num(L, "lam", in.lam) &&
                      json_num(L, "q2", in.q2) && json_num(L, "t0", in.t0);
        if (!parsed || run_id != m.run_id) {
            std::printf("line %" PRIu64 ": unreadable or from another run\n", lines);
            ++bad;
            continue;
        }
        double lam0, dlam;
        bool grid_ok = case_grid(m, in, lam0, dlam) && bits_of(lam0) == lb && bits_of(dlam) == db;
        Trajectory ref = run_reference(in, m.S, of_bits(lb), of_bits(db));
        bool ok = grid_ok;
        if (succ == "true") {
            // The reference data hashed against itself gives the stored roots.
            Trajectory same = ref;
            CaseResult r = compare_case(m, dir, id, ref, same, false);
            ok = ok && r.success && hex(r.case_root) == root;
        } else {
            // A failing case must have its window, whose reference half is the reference data.
            std::string ff, fname;
            uint64_t idx = 0;
            ok = ok && json_raw(L, "first_fail", ff);
            if (ff == "null") {
                // Failed on the invariants or on quantisation: no window to check.
            } else if (ok && json_raw(L, "field", fname) && json_u64(L, "index", idx) &&
                       gkv_field_index(fname.c_str()) >= 0 && idx < m.S) {
                int f = gkv_field_index(fname.c_str());
                uint64_t seg = (idx / kSeg) * kSeg, n = std::min(kSeg, m.S - seg), ws, we;
                gkv_fail_window_bounds(seg, idx - seg, n, kWindow, &ws, &we);
                std::vector<double> a(ref.f[f].begin() + seg, ref.f[f].begin() + seg + n);
                if (f == 3) gkv_unwrap(a.data(), n);
                std::vector<double> wr(we - ws), wp(we - ws);
                ok = gkv_load_fail_window(dir.c_str(), id, f, ws, we, wr.data(), wp.data()) == 0;
                for (uint64_t i = 0; ok && i < we - ws; ++i) ok = bits_of(wr[i]) == bits_of(a[ws - seg + i]);
            } else {
                ok = false;
            }
        }
        if (!ok) {
            std::printf("case %" PRIu64 ": MISMATCH%s\n", id, grid_ok ? "" : " (grid)");
            ++bad;
        }
    }
    std::printf("audited %" PRIu64 " ledger lines: %" PRIu64 " verified, %" PRIu64 " mismatched\n", lines,
                lines - bad, bad);
    return bad ? 2 : 0;
}

int cmd_diff(int argc, char** argv) {
    if (argc < 2 || argv[0][0] == '-' || argv[1][0] == '-') {
        std::fprintf(stderr, "usage: gkval diff <run-id> <case> [field]\n");
        return 1;
    }
    std::string dir = run_dir_of(argc, argv, argv[0]);
    uint64_t id = std::strtoull(argv[1], nullptr, 10);
    int want = -1;
    if (argc > 2 && argv[2][0] != '-') {
        want = gkv_field_index(argv[2]);
        if (want < 0) {
            std::fprintf(stderr, "gkval diff: unknown field %s\n", argv[2]);
            return 1;
        }
    }
    std::string wdir = dir + "/fail_windows/" + std::to_string(id);
    DIR* d = opendir(wdir.c_str());
    int shown = 0;
    if (d) {
        while (dirent* e = readdir(d)) {
            char fname[32];
            unsigned long long s, en;
            if (std::sscanf(e->d_name, "%31[a-z]_%llu_%llu.bin", fname, &s, &en) != 3) continue;
            int f = gkv_field_index(fname);
            if (f < 0 || (want >= 0 && f != want) || en <= s) continue;
            std::vector<double> a(en - s), b(en - s);
            if (gkv_load_fail_window(dir.c_str(), id, f, s, en, a.data(), b.data()) != 0) {
                std::printf("%s: unreadable\n", e->d_name);
                continue;
            }
            ++shown;
            std::printf("case %" PRIu64 " field %s samples [%llu, %llu)\n", id, fname, s, en);
            std::printf("%8s %24s %24s %12s %20s\n", "index", "reference", "port", "|diff|", "ulp");
            for (uint64_t i = 0; i < en - s; ++i)
                std::printf("%8llu %24.16e %24.16e %12.3e %20" PRIu64 "\n", s + i, a[i], b[i], std::fabs(a[i] - b[i]),
                            gkv_ulp_distance(a[i], b[i]));
        }
        closedir(d);
    }
    if (!shown) std::printf("no fail windows for case %" PRIu64 "\n", id);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::printf("usage: gkval init|validate|audit|diff ...\n");
        return 1;
    }
    std::string cmd = argv[1];
    if (cmd == "init") return cmd_init(argc - 2, argv + 2);
    if (cmd == "validate") return cmd_validate(argc - 2, argv + 2);
    if (cmd == "audit") return cmd_audit(argc - 2, argv + 2);
    if (cmd == "diff") return cmd_diff(argc - 2, argv + 2);
    std::fprintf(stderr, "gkval: unknown command %s\n", cmd.c_str());
    return 1;
}
