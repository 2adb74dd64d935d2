/*
 * gkval_core.cpp -- GEOKERR validation harness core (TEST INFRASTRUCTURE ONLY).
 *
 * Restates the observable behaviour of the reference's streaming validator
 * core, geokerr_port/validation/gkval_core.c and gkval_io.c, so that runs,
 * ledgers and fail windows written here read like the reference's:
 *
 *   ULP distance      gkval_core.c:236-258   ordered-integer map of IEEE-754
 *                                            doubles; NaN -> UINT64_MAX; equal
 *                                            infinities 0, else UINT64_MAX
 *   acceptance        gkval_core.c:264-299   |a-b| <= atol + rtol max(|a|,|b|)
 *                                            AND ulp(a,b) <= max_ulps
 *   phi unwrap        gkval_core.c:305-323   +-2 pi against the previous sample
 *   quantisation      gkval_core.c:158-228   round-to-nearest-even at fraction
 *                                            bit quant_lsb, carry into the
 *                                            exponent; NaN/Inf rejected
 *   leaf / node hash  gkval_core.c:87-154    "leaf" || run_id || case_id (u64 LE)
 *                                            || field (u32) || start || end ||
 *                                            quantised data; "node" || L || R
 *   Merkle            gkval_core.c:329-380   pairwise, odd node promoted
 *   fail window       gkval_io.c:140-175     u32 magic "GKPW", u32 version 1,
 *                                            u16 field, u64 start, end, size,
 *                                            f64 reference[size], f64 port[size]
 *                                            (packed), in
 *                                            fail_windows/<case>/<field>_<s>_<e>.bin
 *   adaptive grid     gkval_adapters.c:96-140  lambda_max = K T_char over S - 1
 *                                            steps, T_char from the radial /
 *                                            polar periods
 *
 * The reference's leaf/node hash is a placeholder (a 64-bit multiplicative
 * byte hash spread over 32 bytes, gkval_core.c:24-40, standing in for
 * BLAKE3).  Both that placeholder ("placeholder", for ledgers that must match
 * the reference byte for byte) and SHA-256 (FIPS 180-4; "sha256", the default
 * here) are provided over the same domain-separated messages.
 *
 * Host code only, portable C++ (no x86 control registers: the rounding mode
 * is checked with <cfenv>).  Built into liboracle.so.
 */
#include <cerrno>
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

extern "C" void npo_geokerr_estimate_periods(double u0, double mu0, double a, double Lz, double Q2, double* Tr,
                                             double* Tth, int* info);
extern "C" double npo_geokerr_phi_omega(double u0, double mu0, double a, double Lz, double Q2);

namespace {

constexpr uint32_t kFailMagic = 0x474B5057u;  // "GKPW"
constexpr uint32_t kFailVersion = 1;

// ---------------------------------------------------------------------------
// SHA-256 (FIPS 180-4).  The round constants and initial hash are derived at
// first use from their definition -- the first 32 fraction bits of the cube
// roots of the first 64 primes and of the square roots of the first 8 -- by
// exact integer roots, so no table is written out.

using u128 = unsigned __int128;

uint64_t iroot(u128 v, int k) {  // floor(v^(1/k)) for k = 2, 3, v < 2^110
    uint64_t lo = 0, hi = (k == 2) ? (1ull << 56) : (1ull << 37);
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo + 1) / 2;
        u128 p = (u128)mid * mid;
        if (k == 3) p *= mid;
        if (p <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

struct ShaConsts {
    uint32_t K[64], H0[8];
    ShaConsts() {
        int primes[64], n = 0;
        for (int c = 2; n < 64; ++c) {
            bool is_p = true;
            for (int d = 2; d * d <= c; ++d) if (c % d == 0) { is_p = false; break; }
            if (is_p) primes[n++] = c;
        }
        for (int i = 0; i < 64; ++i) K[i] = (uint32_t)iroot((u128)primes[i] << 96, 3);
        for (int i = 0; i < 8; ++i) H0[i] = (uint32_t)iroot((u128)primes[i] << 64, 2);
    }
};

const ShaConsts& sha_consts() {
    static ShaConsts c;
    return c;
}

inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

void sha256(const uint8_t* msg, size_t len, uint8_t out[32]) {
    const ShaConsts& C = sha_consts();
    uint32_t h[8];
    std::memcpy(h, C.H0, sizeof h);
    std::vector<uint8_t> m(msg, msg + len);
    m.push_back(0x80);
    while (m.size() % 64 != 56) m.push_back(0);
    uint64_t bits = (uint64_t)len * 8;
    for (int i = 7; i >= 0; --i) m.push_back((uint8_t)(bits >> (8 * i)));
    for (size_t blk = 0; blk < m.size(); blk += 64) {
        uint32_t w[64];
        for (int i = 0; i < 16; ++i)
            w[i] = (uint32_t)m[blk + 4 * i] << 24 | (uint32_t)m[blk + 4 * i + 1] << 16 |
                   (uint32_t)m[blk + 4 * i + 2] << 8 | m[blk + 4 * i + 3];
        for (int i = 16; i < 64; ++i) {
            uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
            uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
            w[i] = w[i - 16] + s0 + w[i - 7] + s1;
        }
        uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
        for (int i = 0; i < 64; ++i) {
            uint32_t S1 = rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
            uint32_t ch = (e & f) ^ (~e & g);
            uint32_t t1 = hh + S1 + ch + C.K[i] + w[i];
            uint32_t S0 = rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
            uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
            uint32_t t2 = S0 + mj;
            hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
        }
        h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
    }
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 4; ++j) out[4 * i + j] = (uint8_t)(h[i] >> (24 - 8 * j));
}

// The reference's stand-in hash (gkval_core.c:24-40): a 64-bit state seeded
// 0x1234567890ABCDEF, per byte xor then multiply by 2^40 + 0x1B3; output
// byte i is state byte i mod 8.
void placeholder_hash(const uint8_t* msg, size_t len, uint8_t out[32]) {
    uint64_t s = 0x1234567890ABCDEFull;
    for (size_t i = 0; i < len; ++i) {
        s ^= msg[i];
        s *= 0x100000001B3ull;
    }
    for (int i = 0; i < 32; ++i) out[i] = (uint8_t)(s >> (8 * (i % 8)));
}

void digest(int kind, const std::vector<uint8_t>& m, uint8_t out[32]) {
    if (kind == 1) placeholder_hash(m.data(), m.size(), out);
    else sha256(m.data(), m.size(), out);
}

template <class T>
void put(std::vector<uint8_t>& m, T v) {  // little-endian, as the reference's memcpy on LE hosts
    for (size_t i = 0; i < sizeof(T); ++i) m.push_back((uint8_t)((uint64_t)v >> (8 * i)));
}

inline uint64_t bits_of(double x) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
}

inline uint64_t ordered(double x) {
    uint64_t u = bits_of(x);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

const char* kFieldNames[5] = {"u", "mu", "t", "phi", "affine"};

int mkdir_one(const std::string& p) {
    if (mkdir(p.c_str(), 0755) != 0 && errno != EEXIST) return -2;
    return 0;
}

}  // namespace

extern "C" {

// Error codes as gkval_core.h:201-208.
enum { GKV_OK = 0, GKV_EINVAL = -1, GKV_EIO = -2, GKV_EHASH = -3, GKV_EQUANT = -4, GKV_EMEM = -7 };

const char* gkv_field_name(int field) { return (field >= 0 && field < 5) ? kFieldNames[field] : "unknown"; }

int gkv_field_index(const char* s) {
    for (int i = 0; i < 5; ++i)
        if (s && std::strcmp(s, kFieldNames[i]) == 0) return i;
    return -1;
}

void gkv_sha256(const uint8_t* msg, size_t len, uint8_t* out) { sha256(msg, len, out); }

void gkv_placeholder_hash(const uint8_t* msg, size_t len, uint8_t* out) { placeholder_hash(msg, len, out); }

uint64_t gkv_ulp_distance(double a, double b) {
    if (std::isnan(a) || std::isnan(b)) return UINT64_MAX;
    if (std::isinf(a) || std::isinf(b)) return a == b ? 0 : UINT64_MAX;
    if (a == b) return 0;
    uint64_t oa = ordered(a), ob = ordered(b);
    return oa > ob ? oa - ob : ob - oa;
}

int gkv_accept_sample(double a, double b, double atol, double rtol, uint64_t max_ulps) {
    double diff = std::fabs(a - b);
    double mx = std::fmax(std::fabs(a), std::fabs(b));
    bool tol_ok = diff <= atol + rtol * mx;  // false for NaN, as the reference
    return tol_ok && gkv_ulp_distance(a, b) <= max_ulps;
}

// Index of the first rejected sample in [0, n), or -1 when all pass.
int64_t gkv_first_fail(const double* a, const double* b, size_t n, double atol, double rtol, uint64_t max_ulps) {
    for (size_t i = 0; i < n; ++i)
        if (!gkv_accept_sample(a[i], b[i], atol, rtol, max_ulps)) return (int64_t)i;
    return -1;
}

void gkv_unwrap(double* x, size_t n) {
    for (size_t i = 1; i < n; ++i) {
        double d = x[i] - x[i - 1];
        if (d > M_PI) x[i] -= 2.0 * M_PI;
        else if (d < -M_PI) x[i] += 2.0 * M_PI;
    }
}

int gkv_quantize(double x, int quant_lsb, uint64_t* q) {
    if (!q || quant_lsb < 0 || quant_lsb > 52) return GKV_EINVAL;
    uint64_t b = bits_of(x);
    uint64_t e = (b >> 52) & 0x7FF;
    if (e == 0x7FF) return GKV_EQUANT;
    if (quant_lsb == 0) { *q = b; return GKV_OK; }
    uint64_t sign = b & 0x8000000000000000ull, frac = b & 0x000FFFFFFFFFFFFFull;
    uint64_t unit = 1ull << quant_lsb, tail = frac & (unit - 1), kept = frac & ~(unit - 1);
    uint64_t half = unit >> 1;
    if (tail > half || (tail == half && (kept & unit))) {
        kept += unit;
        if (kept >> 52) {          // fraction overflow: next binade
            kept = 0;
            if (++e >= 0x7FF) return GKV_EQUANT;
        }
    }
    *q = sign | (e << 52) | kept;
    return GKV_OK;
}

int gkv_quantize_block(const double* x, size_t n, int quant_lsb, uint64_t* q) {
    for (size_t i = 0; i < n; ++i) {
        int rc = gkv_quantize(x[i], quant_lsb, q + i);
        if (rc) return rc;
    }
    return GKV_OK;
}

// Leaf hash over quantised samples (hash_kind 0 = SHA-256, 1 = placeholder).
void gkv_hash_leaf(int hash_kind, const char* run_id, uint64_t case_id, int field, uint64_t start, uint64_t end,
                   const uint64_t* q, size_t n, uint8_t* out) {
    std::vector<uint8_t> m{'l', 'e', 'a', 'f'};
    m.insert(m.end(), run_id, run_id + std::strlen(run_id));
    put<uint64_t>(m, case_id);
    put<uint32_t>(m, (uint32_t)field);
    put<uint64_t>(m, start);
    put<uint64_t>(m, end);
    for (size_t i = 0; i < n; ++i) put<uint64_t>(m, q[i]);
    digest(hash_kind, m, out);
}

void gkv_hash_node(int hash_kind, const uint8_t* left, const uint8_t* right, uint8_t* out) {
    std::vector<uint8_t> m{'n', 'o', 'd', 'e'};
    m.insert(m.end(), left, left + 32);
    m.insert(m.end(), right, right + 32);
    digest(hash_kind, m, out);
}

// Merkle root of n 32-byte hashes (zero hash for n = 0).
void gkv_merkle(int hash_kind, const uint8_t* hashes, size_t n, uint8_t* out) {
    if (n == 0) { std::memset(out, 0, 32); return; }
    std::vector<uint8_t> lvl(hashes, hashes + 32 * n);
    while (n > 1) {
        size_t m = (n + 1) / 2;
        for (size_t i = 0; i < m; ++i) {
            uint8_t tmp[32];
            if (2 * i + 1 < n) gkv_hash_node(hash_kind, &lvl[64 * i], &lvl[64 * i + 32], tmp);
            else std::memcpy(tmp, &lvl[64 * i], 32);
            std::memcpy(&lvl[32 * i], tmp, 32);
        }
        n = m;
    }
    std::memcpy(out, lvl.data(), 32);
}

// fail_windows/<case_id>/<field>_<start>_<end>.bin under run_dir.
int gkv_fail_window_path(const char* run_dir, uint64_t case_id, int field, uint64_t start, uint64_t end, char* out,
                         size_t cap) {
    int k = std::snprintf(out, cap, "%s/fail_windows/%llu/%s_%llu_%llu.bin", run_dir, (unsigned long long)case_id,
                          gkv_field_name(field), (unsigned long long)start, (unsigned long long)end);
    return (k > 0 && (size_t)k < cap) ? GKV_OK : GKV_EINVAL;
}

int gkv_save_fail_window(const char* run_dir, uint64_t case_id, int field, uint64_t start, uint64_t end,
                         const double* ref, const double* port) {
    if (!run_dir || !ref || !port || end <= start) return GKV_EINVAL;
    std::string base = std::string(run_dir) + "/fail_windows";
    if (mkdir_one(base) || mkdir_one(base + "/" + std::to_string(case_id))) return GKV_EIO;
    char path[2048];
    if (gkv_fail_window_path(run_dir, case_id, field, start, end, path, sizeof path)) return GKV_EINVAL;
    std::vector<uint8_t> m;
    put<uint32_t>(m, kFailMagic);
    put<uint32_t>(m, kFailVersion);
    put<uint16_t>(m, (uint16_t)field);
    put<uint64_t>(m, start);
    put<uint64_t>(m, end);
    put<uint64_t>(m, end - start);
    size_t n = end - start;
    for (size_t i = 0; i < n; ++i) put<uint64_t>(m, bits_of(ref[i]));
    for (size_t i = 0; i < n; ++i) put<uint64_t>(m, bits_of(port[i]));
    FILE* f = std::fopen(path, "wb");
    if (!f) return GKV_EIO;
    bool ok = std::fwrite(m.data(), 1, m.size(), f) == m.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? GKV_OK : GKV_EIO;
}

int gkv_load_fail_window(const char* run_dir, uint64_t case_id, int field, uint64_t start, uint64_t end,
                         double* ref, double* port) {
    if (!run_dir || !ref || !port || end <= start) return GKV_EINVAL;
    char path[2048];
    if (gkv_fail_window_path(run_dir, case_id, field, start, end, path, sizeof path)) return GKV_EINVAL;
    FILE* f = std::fopen(path, "rb");
    if (!f) return GKV_EIO;
    uint8_t h[34];
    bool ok = std::fread(h, 1, 34, f) == 34;
    auto rd = [&](int off, int nb) {
        uint64_t v = 0;
        for (int i = 0; i < nb; ++i) v |= (uint64_t)h[off + i] << (8 * i);
        return v;
    };
    uint64_t n = end - start;
    ok = ok && rd(0, 4) == kFailMagic && rd(4, 4) == kFailVersion && rd(8, 2) == (uint64_t)field &&
         rd(10, 8) == start && rd(18, 8) == end && rd(26, 8) == n;
    ok = ok && std::fread(ref, 8, n, f) == n && std::fread(port, 8, n, f) == n;
    std::fclose(f);
    return ok ? GKV_OK : GKV_EIO;
}

// Window of `width` samples around local index fail in a segment of n
// samples starting at seg_start (gkval_validator.c:423-458): starts width/2
// before the failure, clipped to the segment.
void gkv_fail_window_bounds(uint64_t seg_start, uint64_t fail, uint64_t n, uint64_t width, uint64_t* start,
                            uint64_t* end) {
    uint64_t s = fail >= width / 2 ? fail - width / 2 : 0;
    uint64_t e = s + width;
    if (e > n) {
        e = n;
        s = e >= width ? e - width : 0;
    }
    *start = seg_start + s;
    *end = seg_start + e;
}

// Per-case lambda grid (gkval_adapters.c:96-140): lam0 = 0 and dlam =
// K T_char / (S - 1), with T_char the radial period for equatorial rays
// (|q2| < 1e-14), else the polar one when u0 = uf, else the larger; a
// failed period estimate counts as T = 1.
int gkv_adaptive_grid(double u0, double mu0, double uf, double a, double lam, double q2, uint64_t S, double K,
                      double* lam0, double* dlam) {
    if (S < 2 || !lam0 || !dlam) return GKV_EINVAL;
    double Tr = -1.0, Tth = -1.0;
    int info = 0;
    npo_geokerr_estimate_periods(u0, mu0, a, lam, q2, &Tr, &Tth, &info);
    if (info != 0) Tr = Tth = 1.0;
    const double eps = 1e-14;
    double Tc;
    if (std::fabs(q2) < eps && Tr > 0) Tc = Tr;
    else if (std::fabs(uf - u0) < eps && Tth > 0) Tc = Tth;
    else if (std::fabs(q2) < eps && std::fabs(uf - u0) < eps) {
        double w = npo_geokerr_phi_omega(u0, mu0, a, lam, q2);
        if (std::fabs(w) < eps) w = 1.0;
        Tc = 2.0 * M_PI / std::fabs(w);
    } else {
        Tc = std::fmax(Tr, Tth);
    }
    if (Tc <= 0.0) Tc = 1.0;
    *lam0 = 0.0;
    *dlam = K * Tc / (double)(S - 1);
    return GKV_OK;
}

// Rounding mode check (the reference's MXCSR check, gkval_core.c:51-85,
// restated portably): round-to-nearest required; fix = 1 sets it.
int gkv_check_fp_env(int fix) {
    if (std::fegetround() == FE_TONEAREST) return GKV_OK;
    if (!fix) return GKV_EIO;
    std::fesetround(FE_TONEAREST);
    return std::fegetround() == FE_TONEAREST ? GKV_OK : GKV_EIO;
}

}  // extern "C"
