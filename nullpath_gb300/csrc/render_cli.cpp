// render_cli.cpp -- the `render` command-line tool over the C ABI
// (include/np_render.h), a drop-in for the reference's render binary.
//
// Flags, defaults, validation messages, exit codes and console lines follow
// render.cu:15-46 (defaults), 397-423 (flags), 431-474 (validation and
// --mode), 523-620 (passes, checkpoints, tone mapping, PPM) and 606-619
// (frames).  Extensions (no counterpart in the reference):
//   --units M|Rs        unit of --rcam (disk edges and escape radius are absolute)
//   --seed N            stratified sub-pixel jitter from seed N (implies --stratified)
//   --stratified        stratified jitter instead of the wanghash pattern
//   --disk-rin isco|R   inner disk edge (isco = prograde ISCO of --mass, --spin)
//   --disk-rout R       outer disk edge
//   --emissivity-q Q    disk emissivity index (j ~ r^-Q)
//   --escape-r R        escape radius
//   --max-steps N       step cap per ray
//   --precision fp64|mixed
//   --integrator rk4|adaptive|rkf78, --rtol X, --atol X
//   --crossing linear|hermite|root
//   --inv-gate X        invariant gate of the rkf78 integrator (|H|, Carter Q)
//   --mode research     FP64, rkf78 at rtol 1e-12 / atol 1e-14, root-found
//                       crossings, invariant gate 1e-12, ZAMO camera and
//                       invariant tracking (explicit flags take precedence)
//   --mode precise      mixed precision, rkf78 at rtol 1e-8 / atol 1e-9 in
//                       compensated FP32, crossings landed on the equator
//                       (Henon steps), FP64 islands (explicit flags take
//                       precedence)
//   --islands N         FP64 island mask of the mixed path (NP_ISLAND_*)
//   --benchmark         the 1280x720, a=0.9 benchmark scene (other flags may follow)
//   --out-raw FILE      float32 mean RGB [3][H][W] and first-crossing radius [H][W]
//   --json FILE         a sidecar with the scene, passes, timings and the
//                       camera azimuth of every frame
//   --accum-out FILE    the accumulator (colour sums, first-crossing radius,
//                       invariant maxima, samples done) at every checkpoint
//   --resume FILE       continue from such a file to --spp-total; the result
//                       is bit-identical to an uninterrupted run with the same
//                       --samples per pass
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "np_render.h"

namespace {

struct Cli {
    np_scene_t scene;
    const char* out_path = "render.ppm";
    int samples = 1;
    int tile_h = 128;
    int frames = 1;
    float turns = 1.0f;
    float phi0_deg = 0.0f;
    const char* out_pat = "frame_%05d.ppm";
    int spp_total = 0;
    int checkpoint_every = 0;
    const char* mode = "balanced";
    float exposure_ev = 0.0f;
    float gamma = 2.2f;
    const char* tonemap = "none";
    const char* bg = "gradient";
    int precision = NP_PREC_FP64;
    const char* out_raw = nullptr;
    const char* json = nullptr;
    const char* accum_out = nullptr;
    const char* resume = nullptr;
    bool rin_isco = false;
    bool integrator_set = false, rtol_set = false, atol_set = false, crossing_set = false, gate_set = false;
    bool precision_set = false;
};

std::string lower(const char* s) {
    std::string o(s ? s : "");
    for (char& c : o) c = (char)std::tolower((unsigned char)c);
    return o;
}

// One %d-like conversion and otherwise only %% (render.cu:375-389).
bool valid_pattern(const char* pat) {
    if (!pat) return false;
    int n = 0;
    for (const char* p = pat; *p; ++p) {
        if (*p != '%') continue;
        ++p;
        if (!*p) return false;
        if (*p == '%') continue;
        if (*p == '-') ++p;
        while (*p >= '0' && *p <= '9') ++p;
        if (*p != 'd') return false;
        ++n;
    }
    return n == 1;
}

bool write_ppm(const char* path, int w, int h, const std::vector<unsigned char>& rgb) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    std::fprintf(f, "P6\n%d %d\n255\n", w, h);
    size_t n = std::fwrite(rgb.data(), 1, rgb.size(), f);
    std::fclose(f);
    return n == rgb.size();
}

// Accumulator file: u32 "NPAC", version 2, W, H, samples done, the scene
// hash (two u32, low first); then float colour sums [3][H][W], first-crossing
// radius [H][W], invariant maxima [3].
struct Accum {
    int w = 0, h = 0, spp = 0;
    uint64_t scene_hash = 0;
    std::vector<float> sum, rc, inv;
};
constexpr unsigned kAccumMagic = 0x4341504eu;   // "NPAC"
constexpr unsigned kAccumVersion = 2u;

// FNV-1a (64-bit) over the fields of the scene that change a sample's colour
// (every field but phi, spp and sample_offset), the precision and the samples
// per pass (the pass split decides the sample order of the sums).  A resumed
// accumulator must come from the same scene, or its sums would mix renders.
uint64_t scene_hash(const np_scene_t& s, int precision, int samples_per_pass) {
    uint64_t h = 1469598103934665603ull;
    auto eat = [&](const void* p, size_t n) {
        const unsigned char* b = (const unsigned char*)p;
        for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ull; }
    };
    auto i32 = [&](int32_t v) { eat(&v, sizeof(v)); };
    auto f64 = [&](double v) { eat(&v, sizeof(v)); };
    i32(s.width); i32(s.height); f64(s.mass); f64(s.spin); f64(s.r_cam); f64(s.theta_deg); f64(s.fov_y_deg);
    i32(s.units); i32(s.camera); i32(s.jitter); i32((int32_t)s.seed); i32(s.integrator); i32(s.max_steps);
    f64(s.step_scale); f64(s.rtol); f64(s.atol); f64(s.escape_r); i32(s.disk_on); i32(s.disk_max_orders);
    f64(s.disk_rin); f64(s.disk_rout); f64(s.emissivity_q); f64(s.disk_gain); i32(s.crossing); i32(s.background);
    f64(s.bg_sigma_deg); f64(s.bg_brightness); i32(s.check_invariants); i32(s.islands); f64(s.inv_gate);
    f64(s.rtol_fp64); i32(s.island_arith);
    i32(precision); i32(samples_per_pass);
    return h;
}

// Writes to path.tmp, flushes and closes it, then renames it over path, so an
// interrupted write never destroys the last complete checkpoint.
bool write_accum(const char* path, const Accum& a) {
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    const unsigned hdr[7] = {kAccumMagic, kAccumVersion, (unsigned)a.w, (unsigned)a.h, (unsigned)a.spp,
                             (unsigned)(a.scene_hash & 0xffffffffu), (unsigned)(a.scene_hash >> 32)};
    bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 &&
              std::fwrite(a.sum.data(), sizeof(float), a.sum.size(), f) == a.sum.size() &&
              std::fwrite(a.rc.data(), sizeof(float), a.rc.size(), f) == a.rc.size() &&
              std::fwrite(a.inv.data(), sizeof(float), a.inv.size(), f) == a.inv.size();
    ok = (std::fflush(f) == 0) && ok;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) { std::remove(tmp.c_str()); return false; }
    return std::rename(tmp.c_str(), path) == 0;
}

// Reads an accumulator file for a w x h frame of the scene with hash `hash`;
// returns an error message or "".
std::string read_accum(const char* path, int w, int h, uint64_t hash, Accum& a) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return std::string("Cannot read ") + path + ".";
    unsigned hdr[7];
    std::string err;
    if (std::fread(hdr, sizeof(unsigned) * 2, 1, f) != 1 || hdr[0] != kAccumMagic) {
        err = std::string(path) + " is not an accumulator file.";
    } else if (hdr[1] != kAccumVersion) {
        err = std::string(path) + " is an accumulator of another version (no scene hash); render it again.";
    } else if (std::fread(hdr + 2, sizeof(unsigned) * 5, 1, f) != 1) {
        err = std::string(path) + " is truncated.";
    } else if ((int)hdr[2] != w || (int)hdr[3] != h) {
        err = std::string(path) + " holds a different image size.";
    } else if ((((uint64_t)hdr[6] << 32) | hdr[5]) != hash) {
        err = std::string(path) + " was rendered from a different scene, precision or --samples; it cannot be resumed.";
    } else {
        const size_t npix = (size_t)w * h;
        a.w = w; a.h = h; a.spp = (int)hdr[4];
        a.sum.resize(3 * npix); a.rc.resize(npix); a.inv.resize(3);
        if (std::fread(a.sum.data(), sizeof(float), a.sum.size(), f) != a.sum.size() ||
            std::fread(a.rc.data(), sizeof(float), a.rc.size(), f) != a.rc.size() ||
            std::fread(a.inv.data(), sizeof(float), a.inv.size(), f) != a.inv.size())
            err = std::string(path) + " is truncated.";
    }
    std::fclose(f);
    return err;
}

bool write_raw(const char* path, int w, int h, int spp, const std::vector<float>& rgb, const std::vector<float>& rc) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    const unsigned hdr[5] = {0x5752504eu /* "NPRW" */, 1u, (unsigned)w, (unsigned)h, (unsigned)spp};
    bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 && std::fwrite(rgb.data(), sizeof(float), rgb.size(), f) == rgb.size() &&
              std::fwrite(rc.data(), sizeof(float), rc.size(), f) == rc.size();
    std::fclose(f);
    return ok;
}

void parse(int argc, char** argv, Cli& c) {
    np_scene_t& s = c.scene;
    for (int i = 1; i < argc; ++i) {
        std::string a(argv[i]);
        auto has = [&]() { return i + 1 < argc; };
        auto f = [&](double& v) { if (has()) v = std::strtod(argv[++i], nullptr); };
        auto fl = [&](float& v) { if (has()) v = std::strtof(argv[++i], nullptr); };
        auto n = [&](int& v) { if (has()) v = std::atoi(argv[++i]); };
        auto str = [&](const char*& v) { if (has()) v = argv[++i]; };
        if (a == "--w" || a == "-w") n(s.width);
        else if (a == "--h" || a == "-h") n(s.height);
        else if (a == "--fov") f(s.fov_y_deg);
        else if (a == "--theta") f(s.theta_deg);
        else if (a == "--mass") f(s.mass);
        else if (a == "--rcam") f(s.r_cam);
        else if (a == "--out") str(c.out_path);
        else if (a == "--samples" || a == "-s") n(c.samples);
        else if (a == "--spp-total") n(c.spp_total);
        else if (a == "--checkpoint-every") n(c.checkpoint_every);
        else if (a == "--spin") f(s.spin);
        else if (a == "--check-invariants") s.check_invariants = 1;
        else if (a == "--tile") n(c.tile_h);
        else if (a == "--frames") n(c.frames);
        else if (a == "--turns") fl(c.turns);
        else if (a == "--phi0") fl(c.phi0_deg);
        else if (a == "--outpat") str(c.out_pat);
        else if (a == "--mode" && has()) c.mode = argv[++i];
        else if (a == "--exposure") fl(c.exposure_ev);
        else if (a == "--gamma") fl(c.gamma);
        else if (a == "--tonemap" && has()) c.tonemap = argv[++i];
        else if (a == "--bg" && has()) c.bg = argv[++i];
        else if (a == "--bg-sigma") f(s.bg_sigma_deg);
        else if (a == "--bg-bright") f(s.bg_brightness);
        else if (a == "--no-disk") s.disk_on = 0;
        else if (a == "--disk-gain") f(s.disk_gain);
        else if (a == "--disk-max-orders") n(s.disk_max_orders);
        // extensions
        else if (a == "--benchmark") np_scene_benchmark(&s);
        else if (a == "--units" && has()) { std::string u = lower(argv[++i]); s.units = u == "m" ? NP_UNITS_M : NP_UNITS_RS; }
        else if (a == "--seed") { int v = 0; n(v); s.seed = (uint32_t)v; s.jitter = NP_JITTER_STRATIFIED; }
        else if (a == "--stratified") s.jitter = NP_JITTER_STRATIFIED;
        else if (a == "--disk-rin" && has()) {
            std::string v = lower(argv[++i]);
            if (v == "isco") c.rin_isco = true;
            else { c.rin_isco = false; s.disk_rin = std::strtod(v.c_str(), nullptr); }
        }
        else if (a == "--disk-rout") f(s.disk_rout);
        else if (a == "--emissivity-q") f(s.emissivity_q);
        else if (a == "--escape-r") f(s.escape_r);
        else if (a == "--max-steps") n(s.max_steps);
        else if (a == "--precision" && has()) {
            c.precision = lower(argv[++i]) == "mixed" ? NP_PREC_MIXED : NP_PREC_FP64;
            c.precision_set = true;
        }
        else if (a == "--integrator" && has()) {
            std::string v = lower(argv[++i]);
            s.integrator = v == "adaptive" ? NP_INTEG_ADAPTIVE : v == "rkf78" ? NP_INTEG_RKF78 : NP_INTEG_RK4;
            c.integrator_set = true;
        }
        else if (a == "--rtol") { f(s.rtol); c.rtol_set = true; }
        else if (a == "--atol") { f(s.atol); c.atol_set = true; }
        else if (a == "--inv-gate") { f(s.inv_gate); c.gate_set = true; }
        else if (a == "--crossing" && has()) {
            std::string v = lower(argv[++i]);
            s.crossing = v == "hermite" ? NP_CROSS_HERMITE : v == "root" ? NP_CROSS_ROOT : NP_CROSS_LINEAR;
            c.crossing_set = true;
        }
        else if (a == "--islands") n(s.islands);
        else if (a == "--out-raw") str(c.out_raw);
        else if (a == "--json") str(c.json);
        else if (a == "--accum-out") str(c.accum_out);
        else if (a == "--resume") str(c.resume);
    }
}

}  // namespace

int main(int argc, char** argv) {
    Cli c;
    np_scene_defaults(&c.scene);
    parse(argc, argv, c);
    np_scene_t& s = c.scene;

    if (s.width <= 0 || s.height <= 0) { std::fprintf(stderr, "Invalid image dimensions.\n"); return 1; }
    if (c.tile_h <= 0) { std::fprintf(stderr, "Invalid tile height.\n"); return 1; }
    if (c.samples <= 0) { std::fprintf(stderr, "Invalid samples per pixel.\n"); return 1; }
    if (c.spp_total < 0) { std::fprintf(stderr, "Invalid total spp.\n"); return 1; }
    if (c.frames <= 0) { std::fprintf(stderr, "Invalid frame count.\n"); return 1; }
    if (s.mass <= 0.0 || s.r_cam <= 0.0) { std::fprintf(stderr, "Invalid mass or camera radius.\n"); return 1; }
    if (std::fabs(s.spin) >= 1.0) { std::fprintf(stderr, "Spin must satisfy |a/M| < 1.\n"); return 1; }
    if (s.fov_y_deg <= 0.0 || s.fov_y_deg >= 179.0) {
        std::fprintf(stderr, "Invalid FOV; expected (0, 179) degrees.\n");
        return 1;
    }
    // --mode (render.cu:468-474): accurate = adaptive step doubling, ZAMO
    // camera and invariant tracking; fast and balanced = fixed RK4, static camera
    const std::string mode = lower(c.mode);
    if (mode == "accurate") {
        if (!c.integrator_set) s.integrator = NP_INTEG_ADAPTIVE;
        s.camera = NP_CAMERA_ZAMO;
        s.check_invariants = 1;
    } else if (mode == "research") {
        if (!c.precision_set) c.precision = NP_PREC_FP64;
        if (!c.integrator_set) s.integrator = NP_INTEG_RKF78;
        if (!c.rtol_set) s.rtol = 1e-12;
        if (!c.atol_set) s.atol = 1e-14;
        if (!c.crossing_set) s.crossing = NP_CROSS_ROOT;
        if (!c.gate_set) s.inv_gate = 1e-12;
        s.camera = NP_CAMERA_ZAMO;
        s.check_invariants = 1;
    } else if (mode == "precise") {
        if (!c.precision_set) c.precision = NP_PREC_MIXED;
        if (!c.integrator_set) s.integrator = NP_INTEG_RKF78;
        if (!c.rtol_set) s.rtol = 1e-8;
        if (!c.atol_set) s.atol = 1e-9;
        if (!c.crossing_set) s.crossing = NP_CROSS_ROOT;
    }
    if (c.precision == NP_PREC_MIXED && mode == "research") {
        std::fprintf(stderr, "Research mode needs --precision fp64.\n");
        return 1;
    }
    if (c.precision == NP_PREC_MIXED && s.inv_gate > 0.0) {
        std::fprintf(stderr, "The invariant gate needs --precision fp64.\n");
        return 1;
    }
    if (c.precision == NP_PREC_MIXED && s.crossing == NP_CROSS_ROOT && s.integrator != NP_INTEG_RKF78) {
        std::fprintf(stderr, "Root crossings on --precision mixed need --integrator rkf78.\n");
        return 1;
    }
    s.background = lower(c.bg) == "point" ? NP_BG_POINT : NP_BG_GRADIENT;
    if (c.rin_isco) s.disk_rin = np_isco_radius(s.mass, s.spin);
    const bool reinhard = lower(c.tonemap) == "reinhard";
    if (np_scene_validate(&s) != NP_OK) { std::fprintf(stderr, "%s\n", np_last_error()); return 1; }
    if ((c.resume || c.accum_out) && c.frames > 1) {
        std::fprintf(stderr, "--resume and --accum-out need a single frame.\n");
        return 1;
    }
    Accum resumed;
    if (c.resume) {
        std::string err = read_accum(c.resume, s.width, s.height, scene_hash(s, c.precision, c.samples), resumed);
        if (!err.empty()) { std::fprintf(stderr, "%s\n", err.c_str()); return 1; }
    }

    np_frame_t* fr = np_frame_create(s.width, s.height, nullptr);
    if (!fr) { std::fprintf(stderr, "%s\n", np_last_error()); return 1; }
    const size_t npix = (size_t)s.width * s.height;
    std::vector<unsigned char> rgb8(3 * npix);
    double kernel_ms = 0.0;
    unsigned long long rays = 0, steps = 0;
    int passes_done = 0;

    auto render_one = [&](double phi_deg, const char* path) -> bool {
        const int total = c.spp_total > 0 ? c.spp_total : c.samples;
        const int batch = c.samples > 1 ? c.samples : 1;
        np_frame_reset(fr);
        if (c.resume && np_frame_load(fr, resumed.sum.data(), resumed.rc.data(), resumed.inv.data(),
                                      resumed.spp) != NP_OK) {
            std::fprintf(stderr, "%s\n", np_last_error());
            return false;
        }
        const int remaining = std::max(0, total - np_frame_spp(fr));
        const int passes = std::max(1, (remaining + batch - 1) / batch);
        np_scene_t ps = s;
        ps.phi_deg = phi_deg;
        for (int p = 0; p < passes; ++p) {
            if (remaining == 0) {
                // the accumulator already holds the requested samples: write it out
                if (np_frame_spp(fr) <= 0) { std::fprintf(stderr, "Nothing to render.\n"); return false; }
            } else {
                ps.spp = std::min(batch, total - np_frame_spp(fr));
                np_render_stats_t st{};
                if (np_frame_add_pass(fr, &ps, c.precision, &st) != NP_OK) {
                    std::fprintf(stderr, "%s\n", np_last_error());
                    return false;
                }
                kernel_ms += st.kernel_ms + st.init_ms;
                rays += st.rays; steps += st.steps;
                ++passes_done;
            }
            const bool ckpt = p == passes - 1 || (c.checkpoint_every > 0 && (p + 1) % c.checkpoint_every == 0);
            if (!ckpt) continue;
            if (c.accum_out) {
                Accum a;
                a.w = s.width; a.h = s.height;
                a.scene_hash = scene_hash(s, c.precision, c.samples);
                a.sum.resize(3 * npix); a.rc.resize(npix); a.inv.resize(3);
                if (np_frame_save(fr, a.sum.data(), a.rc.data(), a.inv.data(), &a.spp) != NP_OK ||
                    !write_accum(c.accum_out, a)) {
                    std::fprintf(stderr, "Failed to write %s\n", c.accum_out);
                    return false;
                }
            }
            if (np_frame_tonemap(fr, c.exposure_ev, c.gamma, reinhard ? 1 : 0, rgb8.data()) != NP_OK) {
                std::fprintf(stderr, "%s\n", np_last_error());
                return false;
            }
            if (!write_ppm(path, s.width, s.height, rgb8)) { std::fprintf(stderr, "Failed to write %s\n", path); return false; }
            if (s.check_invariants) {
                float inv[3] = {0, 0, 0};
                np_frame_read(fr, nullptr, nullptr, inv);
                std::printf("[checkpoint] %s @ %d spp  H|max=%.3e  dE/E|max=%.3e  dL/L|max=%.3e\n", path, np_frame_spp(fr),
                            inv[0], inv[1], inv[2]);
            } else {
                std::printf("[checkpoint] %s @ %d spp\n", path, np_frame_spp(fr));
            }
        }
        if (c.out_raw) {
            std::vector<float> mean(3 * npix), rc(npix);
            if (np_frame_read(fr, mean.data(), rc.data(), nullptr) != NP_OK ||
                !write_raw(c.out_raw, s.width, s.height, np_frame_spp(fr), mean, rc)) {
                std::fprintf(stderr, "Failed to write %s\n", c.out_raw);
                return false;
            }
        }
        return true;
    };

    int rc = 0;
    std::vector<double> frame_phi;   // camera azimuth of each frame, for the sidecar
    if (c.frames <= 1) {
        if (!render_one(c.phi0_deg, c.out_path)) rc = 1;
        else std::printf("Wrote %s\n", c.out_path);
    } else if (!valid_pattern(c.out_pat)) {
        std::fprintf(stderr, "Invalid --outpat (expected a single %%d-like specifier).\n");
        rc = 1;
    } else {
        for (int i = 0; i < c.frames && rc == 0; ++i) {
            const float t = (float)i / (float)c.frames;
            const double phi = c.phi0_deg + 360.0 * c.turns * t;
            frame_phi.push_back(phi);
            char path[512];
            std::snprintf(path, sizeof(path), c.out_pat, i);
            if (!render_one(phi, path)) rc = 1;
        }
        if (rc == 0) std::printf("Wrote %d frames matching pattern %s\n", c.frames, c.out_pat);
    }
    if (rc == 0 && c.json) {
        FILE* f = std::fopen(c.json, "w");
        if (f) {
            std::fprintf(f,
                         "{\"width\": %d, \"height\": %d, \"spp\": %d, \"frames\": %d, \"passes\": %d, \"mass\": %.17g, "
                         "\"spin\": %.17g, \"r_cam\": %.17g, \"theta_deg\": %.17g, \"fov_y_deg\": %.17g, \"units\": \"%s\", "
                         "\"precision\": \"%s\", \"integrator\": \"%s\", \"integrator_order\": %d, "
                         "\"mode\": \"%s\", \"crossing\": \"%s\", \"rtol\": %.17g, \"atol\": %.17g, "
                         "\"inv_gate\": %.17g, \"camera\": \"%s\", \"seed\": %u, \"jitter\": %d, "
                         "\"rays\": %llu, \"steps\": %llu, "
                         "\"kernel_ms\": %.6f, \"rays_per_s\": %.6g, \"frame_phi_deg\": [",
                         s.width, s.height, np_frame_spp(fr), c.frames, passes_done, s.mass, s.spin, s.r_cam, s.theta_deg,
                         s.fov_y_deg, s.units == NP_UNITS_M ? "M" : "Rs", c.precision == NP_PREC_MIXED ? "mixed" : "fp64",
                         s.integrator == NP_INTEG_ADAPTIVE ? "adaptive" : s.integrator == NP_INTEG_RKF78 ? "rkf78" : "rk4",
                         s.integrator == NP_INTEG_RKF78 ? 8 : 4, mode.c_str(),
                         s.crossing == NP_CROSS_ROOT ? "root" : s.crossing == NP_CROSS_HERMITE ? "hermite" : "linear",
                         s.rtol, s.atol, s.inv_gate, s.camera == NP_CAMERA_ZAMO ? "zamo" : "static", s.seed, s.jitter,
                         rays, steps, kernel_ms, kernel_ms > 0 ? rays / (kernel_ms * 1e-3) : 0.0);
            if (frame_phi.empty()) frame_phi.push_back(c.phi0_deg);
            for (size_t i = 0; i < frame_phi.size(); ++i) std::fprintf(f, "%s%.17g", i ? ", " : "", frame_phi[i]);
            std::fprintf(f, "]}\n");
            std::fclose(f);
        }
    }
    np_frame_destroy(fr);
    return rc;
}
