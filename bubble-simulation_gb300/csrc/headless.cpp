// bubble-sim: the windowless driver, built on the C ABI alone.
//
// Mirrors the reference's command line (src/config.rs:193-297, validation
// src/config.rs:333-360, dispatch src/main.rs:27-34) and its headless run
// (src/headless.rs:23-150): the same banner, table, drift baseline (first
// report after every bubble is in), R_eq and throughput line.
// --screenshot renders one frame with the CUDA volume renderer and writes
// it as a PNG (src/capture.rs:19-117, called from src/headless.rs:102-114).
// The interactive window is not part of this build and is rejected with an
// error.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bubble.h"
#include "../../include/bubble_checkpoint.h"
#include "../../include/bubble_render.h"

namespace {

struct Args {
    uint32_t grid[3] = {192, 192, 192};
    float lambda = 0.5f, eps_ratio = 0.3f, alpha = 0.1f, eta = 0.3f, cfl = 0.2f;
    float seed_factor = 1.15f;
    bool has_seed_radius = false;
    float seed_radius = 0.0f;
    long long bubbles = 12;
    int nucleation = BUBBLE_NUCLEATION_EXPONENTIAL;
    float nucleation_duration = 60.0f;
    unsigned long long seed = 1;
    long long steps_per_frame = 2;
    bool has_headless = false;
    unsigned long long headless = 0;
    bool has_report_every = false;
    unsigned long long report_every = 0;
    std::string screenshot;
    uint32_t screenshot_size[2] = {1280, 960};
    std::string save_checkpoint, resume;
    int field = BUBBLE_FIELD_KINETIC;
    int precision = BUBBLE_PRECISION_SINGLE;
    int math = BUBBLE_MATH_FAST;
};

[[noreturn]] void die(const std::string &msg, int code = 2) {
    std::fprintf(stderr, "error: %s\n", msg.c_str());
    std::exit(code);
}

bool parse_grid(const std::string &s, uint32_t out[3]) {
    std::vector<long long> nums;
    size_t pos = 0;
    while (pos <= s.size()) {
        size_t c = s.find(',', pos);
        std::string part = s.substr(pos, c == std::string::npos ? std::string::npos : c - pos);
        size_t a = part.find_first_not_of(" \t"), b = part.find_last_not_of(" \t");
        if (a == std::string::npos) return false;
        part = part.substr(a, b - a + 1);
        char *end = nullptr;
        const long long v = std::strtoll(part.c_str(), &end, 10);
        if (*end != '\0' || v < 0 || v > 0xffffffffLL) return false;
        nums.push_back(v);
        if (c == std::string::npos) break;
        pos = c + 1;
    }
    if (nums.size() == 1) {
        out[0] = out[1] = out[2] = (uint32_t)nums[0];
        return true;
    }
    if (nums.size() == 3) {
        for (int k = 0; k < 3; ++k) out[k] = (uint32_t)nums[k];
        return true;
    }
    return false;
}

float parse_f(const char *v, const char *flag) {
    char *end = nullptr;
    const float f = std::strtof(v, &end);
    if (!v[0] || *end) die(std::string("invalid value '") + v + "' for '" + flag + "'");
    return f;
}
unsigned long long parse_u(const char *v, const char *flag) {
    char *end = nullptr;
    const unsigned long long u = std::strtoull(v, &end, 10);
    if (!v[0] || *end || v[0] == '-') die(std::string("invalid value '") + v + "' for '" + flag + "'");
    return u;
}

void usage() {
    std::printf(
        "bubble-sim: GB300 lattice simulation of bubble nucleation and growth\n\n"
        "Usage: bubble-sim [OPTIONS] --headless N\n\n"
        "  --grid N|A,B,C            lattice size [default: 192]\n"
        "  --lambda F                quartic coupling [default: 0.5]\n"
        "  --eps-ratio F             vacuum energy split [default: 0.3]\n"
        "  --alpha F                 transition strength [default: 0.1]\n"
        "  --eta F                   wall friction [default: 0.3]\n"
        "  --cfl F                   Courant number, <= 0.5 [default: 0.2]\n"
        "  --seed-factor F           seed radius in units of R_c [default: 1.15]\n"
        "  --seed-radius CELLS       fixed seed radius in cells\n"
        "  --bubbles N               bubbles to seed [default: 12]\n"
        "  --nucleation MODE         simultaneous|exponential|centre|uniform [default: exponential]\n"
        "  --nucleation-duration F   time over which nucleation completes [default: 60]\n"
        "  --seed N                  placement seed [default: 1]\n"
        "  --steps-per-frame N       steps per frame [default: 2]\n"
        "  --headless N              run N steps and print diagnostics\n"
        "  --report-every K          report interval [default: max(N/20, 1)]\n"
        "  --precision MODE          single|mixed|double|perturbation [default: single]\n"
        "  --math MODE               fast|strict [default: fast]\n"
        "  --field F                 phi|speed|temperature|kinetic, for --screenshot [default: kinetic]\n"
        "  --screenshot PATH         render one frame to this PNG and exit\n"
        "  --screenshot-size WxH     resolution of --screenshot [default: 1280x960]\n"
        "  --no-vsync                accepted for compatibility; no effect headless\n"
        "  --save-checkpoint PATH    write the final state to a checkpoint file\n"
        "  --resume PATH             continue from a checkpoint (its grid, model and schedule;\n"
        "                            --precision/--math must match its FP32/FP64 layout)\n");
}

bool parse_size(const std::string &s, uint32_t out[2], std::string &msg);

Args parse(int argc, char **argv) {
    Args a;
    for (int i = 1; i < argc; ++i) {
        std::string f = argv[i];
        std::string val;
        bool has_eq = false;
        const size_t eq = f.find('=');
        if (f.rfind("--", 0) == 0 && eq != std::string::npos) {
            val = f.substr(eq + 1);
            f = f.substr(0, eq);
            has_eq = true;
        }
        auto next = [&]() -> const char * {
            if (has_eq) return val.c_str();
            if (i + 1 >= argc) die("a value is required for '" + f + "'");
            return argv[++i];
        };
        if (f == "--help" || f == "-h") {
            usage();
            std::exit(0);
        } else if (f == "--grid") {
            const char *v = next();
            if (!parse_grid(v, a.grid)) die(std::string("`") + v + "` is not a lattice size");
        } else if (f == "--lambda") a.lambda = parse_f(next(), "--lambda");
        else if (f == "--eps-ratio") a.eps_ratio = parse_f(next(), "--eps-ratio");
        else if (f == "--alpha") a.alpha = parse_f(next(), "--alpha");
        else if (f == "--eta") a.eta = parse_f(next(), "--eta");
        else if (f == "--cfl") a.cfl = parse_f(next(), "--cfl");
        else if (f == "--seed-factor") a.seed_factor = parse_f(next(), "--seed-factor");
        else if (f == "--seed-radius") {
            a.has_seed_radius = true;
            a.seed_radius = parse_f(next(), "--seed-radius");
        } else if (f == "--bubbles") a.bubbles = (long long)parse_u(next(), "--bubbles");
        else if (f == "--nucleation") {
            const std::string m = next();
            if (m == "simultaneous") a.nucleation = BUBBLE_NUCLEATION_SIMULTANEOUS;
            else if (m == "exponential") a.nucleation = BUBBLE_NUCLEATION_EXPONENTIAL;
            else if (m == "centre" || m == "center") a.nucleation = BUBBLE_NUCLEATION_CENTRE;
            else if (m == "uniform") a.nucleation = BUBBLE_NUCLEATION_UNIFORM;
            else die("invalid value '" + m + "' for '--nucleation'");
        } else if (f == "--nucleation-duration")
            a.nucleation_duration = parse_f(next(), "--nucleation-duration");
        else if (f == "--seed") a.seed = parse_u(next(), "--seed");
        else if (f == "--steps-per-frame") a.steps_per_frame = (long long)parse_u(next(), "--steps-per-frame");
        else if (f == "--headless") {
            a.has_headless = true;
            a.headless = parse_u(next(), "--headless");
        } else if (f == "--report-every") {
            a.has_report_every = true;
            a.report_every = parse_u(next(), "--report-every");
        } else if (f == "--screenshot") a.screenshot = next();
        else if (f == "--screenshot-size") {
            const std::string v = next();
            std::string msg;
            if (!parse_size(v, a.screenshot_size, msg))
                die("invalid value '" + v + "' for '--screenshot-size <SCREENSHOT_SIZE>': " + msg);
        } else if (f == "--save-checkpoint") a.save_checkpoint = next();
        else if (f == "--resume") a.resume = next();
        else if (f == "--field") {
            const std::string m = next();
            if (m == "phi") a.field = BUBBLE_FIELD_PHI;
            else if (m == "speed") a.field = BUBBLE_FIELD_SPEED;
            else if (m == "temperature") a.field = BUBBLE_FIELD_TEMPERATURE;
            else if (m == "kinetic") a.field = BUBBLE_FIELD_KINETIC;
            else die("invalid value '" + m + "' for '--field'");
        }
        else if (f == "--no-vsync") {
        } else if (f == "--precision") {
            const std::string m = next();
            if (m == "single") a.precision = BUBBLE_PRECISION_SINGLE;
            else if (m == "mixed") a.precision = BUBBLE_PRECISION_MIXED;
            else if (m == "double") a.precision = BUBBLE_PRECISION_DOUBLE;
            else if (m == "perturbation") a.precision = BUBBLE_PRECISION_PERTURBATION;
            else die("invalid value '" + m + "' for '--precision'");
        } else if (f == "--math") {
            const std::string m = next();
            if (m == "fast") a.math = BUBBLE_MATH_FAST;
            else if (m == "strict") a.math = BUBBLE_MATH_STRICT;
            else die("invalid value '" + m + "' for '--math'");
        } else {
            die("unexpected argument '" + f + "'");
        }
    }
    return a;
}

// parse_size (src/config.rs:181-192): WIDTHxHEIGHT (or X), both positive.
bool parse_size(const std::string &s, uint32_t out[2], std::string &msg) {
    const size_t c = s.find_first_of("xX");
    if (c == std::string::npos) {
        msg = "`" + s + "` is not a size; expected WIDTHxHEIGHT";
        return false;
    }
    const std::string parts[2] = {s.substr(0, c), s.substr(c + 1)};
    const char *what[2] = {"width", "height"};
    for (int k = 0; k < 2; ++k) {
        std::string p = parts[k];
        const size_t a = p.find_first_not_of(" \t"), b = p.find_last_not_of(" \t");
        p = a == std::string::npos ? std::string() : p.substr(a, b - a + 1);
        char *end = nullptr;
        const unsigned long long v = p.empty() ? 0 : std::strtoull(p.c_str(), &end, 10);
        if (p.empty() || *end != '\0' || p[0] == '-' || p[0] == '+' || v > 0xffffffffULL) {
            msg = std::string(what[k]) + ": invalid digit found in string";
            return false;
        }
        if (v == 0) {
            msg = std::string(what[k]) + " must be positive";
            return false;
        }
        out[k] = (uint32_t)v;
    }
    return true;
}

bubble_model model_of(const Args &a) {
    bubble_model m;
    bubble_model_default(&m);
    m.lambda = a.lambda;
    m.eps_ratio = a.eps_ratio;
    m.alpha = a.alpha;
    m.eta = a.eta;
    m.cfl = a.cfl;
    if (a.has_seed_radius) {
        m.seed_kind = BUBBLE_SEED_CELLS;
        m.seed_value = a.seed_radius;
    } else {
        m.seed_kind = BUBBLE_SEED_CRITICAL;
        m.seed_value = a.seed_factor;
    }
    return m;
}

// Config::validate (src/config.rs:333-360).
void validate(const Args &a) {
    const bubble_model m = model_of(a);
    if (bubble_model_validate(&m) != BUBBLE_OK) die(bubble_last_error(), 1);
    if (a.bubbles == 0) die("--bubbles must be at least 1", 1);
    if (a.steps_per_frame == 0) die("--steps-per-frame must be at least 1", 1);
    if (a.nucleation_duration <= 0.0f) die("--nucleation-duration must be positive", 1);
    bubble_derived d;
    bubble_model_derived(&m, &d);
    if (d.wall_width < 2.0f) {
        char buf[256];
        std::snprintf(buf, sizeof(buf),
                      "lambda = %g gives a wall only %.2f cells thick, which the lattice cannot "
                      "resolve; use lambda <= %.2f",
                      (double)a.lambda, (double)d.wall_width, 2.0);
        die(buf, 1);
    }
    for (int k = 0; k < 3; ++k)
        if (a.grid[k] < 8)
            die("grid axis " + std::to_string(k) + " is " + std::to_string(a.grid[k]) +
                    "; the 5-point stencil needs at least 8 cells",
                1);
}

// Rust's `{:.3e}`: mantissa with 3 decimals, exponent without '+' or
// leading zeros ("4.587e-5").
std::string rust_exp3(float v) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.3e", (double)v);
    std::string s(buf);
    const size_t e = s.find('e');
    if (e == std::string::npos) return s;
    std::string mant = s.substr(0, e);
    std::string ex = s.substr(e + 1);
    bool neg = false;
    size_t p = 0;
    if (p < ex.size() && (ex[p] == '+' || ex[p] == '-')) {
        neg = ex[p] == '-';
        ++p;
    }
    while (p + 1 < ex.size() && ex[p] == '0') ++p;
    return mant + "e" + (neg ? "-" : "") + ex.substr(p);
}

std::string pad_left(const std::string &s, size_t w) {
    return s.size() >= w ? s : std::string(w - s.size(), ' ') + s;
}

int run(const Args &a, unsigned long long steps, unsigned long long every) {
    bubble_spec spec;
    bubble_spec_default(&spec);
    spec.model = model_of(a);
    for (int k = 0; k < 3; ++k) spec.grid[k] = a.grid[k];
    spec.nucleation = a.nucleation;
    spec.bubbles = (uint64_t)a.bubbles;
    spec.nucleation_duration = a.nucleation_duration;
    spec.seed = a.seed;
    spec.precision = a.precision;
    spec.math = a.math;
    bubble_sim *sim = nullptr;
    if (!a.resume.empty()) {
        // the checkpoint's grid, model, schedule and clock; this run's arithmetic
        bubble_spec saved;
        if (bubble_checkpoint_spec(a.resume.c_str(), &saved) != BUBBLE_OK) die(bubble_last_error(), 1);
        saved.precision = spec.precision;
        saved.math = spec.math;
        spec = saved;
        if (bubble_create(&spec, &sim) != BUBBLE_OK)
            die(std::string("failed to create the simulation: ") + bubble_last_error(), 1);
        if (bubble_checkpoint_restore(sim, a.resume.c_str()) != BUBBLE_OK) die(bubble_last_error(), 1);
    } else if (bubble_create(&spec, &sim) != BUBBLE_OK) {
        die(std::string("failed to create the simulation: ") + bubble_last_error(), 1);
    }
    bubble_vram_info vi;
    if (bubble_vram_query(&vi) == BUBBLE_OK)
        std::printf("adapter: CUDA device (%.1f GB)\n", (double)vi.capacity / 1e9);
    bubble_derived d;
    bubble_model_derived(&spec.model, &d);
    std::printf("lattice %ux%ux%u = %.2f M cells | %.2f GB | dt = %.3f\n", spec.grid[0], spec.grid[1],
                spec.grid[2], (double)bubble_cell_count(sim) / 1e6,
                (double)bubble_device_memory_bytes(sim) / 1e9, (double)d.dt);
    std::printf("wall %.2f cells | R_c %.1f cells | sigma %.4f | eps %.4f | e_ref %.4f\n",
                (double)d.wall_width, (double)d.critical_radius, (double)d.surface_tension,
                (double)d.eps, (double)d.e_ref);
    if (steps > 0)
        std::printf("\n%10s %10s %10s %10s %11s %11s %10s\n", "step", "time", "broken", "R_eq",
                    "max|v|", "K", "E/E0");
    bool have_baseline = false;
    double baseline = 0.0;
    unsigned long long done = 0;
    const auto start = std::chrono::steady_clock::now();
    while (done < steps) {
        const unsigned long long chunk = every < steps - done ? every : steps - done;
        if (bubble_advance(sim, chunk) != BUBBLE_OK) die(bubble_last_error(), 1);
        done += chunk;
        bubble_diag dg;
        const int rc = bubble_diagnostics(sim, &dg);
        if (rc == BUBBLE_ERR_NONFINITE || !std::isfinite(dg.mean_energy) || !std::isfinite(dg.max_velocity)) {
            std::fprintf(stderr,
                         "error: the solution blew up at step %llu (non-finite diagnostics); "
                         "reduce --cfl or --alpha\n",
                         done);
            bubble_destroy(sim);
            return 1;
        }
        if (rc != BUBBLE_OK) die(bubble_last_error(), 1);
        if (!have_baseline && bubble_remaining_bubbles(sim) == 0) {
            have_baseline = true;
            baseline = dg.mean_energy_f64;
        }
        std::string ratio = "-";
        if (have_baseline) {
            char b[64];
            std::snprintf(b, sizeof(b), "%.6f", dg.mean_energy_f64 / baseline);
            ratio = b;
        }
        const float cells = (float)bubble_cell_count(sim);
        const float volume = dg.broken_fraction * cells;
        const float r_eq = std::cbrt(volume * 3.0f / (4.0f * 3.14159265358979323846f));
        std::printf("%10llu %10.1f %9.2f%% %10.1f %11.4f %s %s\n", (unsigned long long)bubble_steps(sim),
                    (double)bubble_time(sim),
                    100.0 * (double)dg.broken_fraction, (double)r_eq, (double)dg.max_velocity,
                    pad_left(rust_exp3(dg.kinetic_fraction), 11).c_str(), pad_left(ratio, 10).c_str());
        std::fflush(stdout);
    }
    const double elapsed =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    if (steps > 0) {
        const double cell_steps = (double)steps * (double)bubble_cell_count(sim);
        std::printf("\n%llu steps in %.2f s  (%.1f steps/s, %.2f G cell-updates/s)\n", steps, elapsed,
                    (double)steps / elapsed, cell_steps / elapsed / 1e9);
    }
    if (!a.save_checkpoint.empty()) {
        if (bubble_checkpoint_save(sim, a.save_checkpoint.c_str()) != BUBBLE_OK) {
            const std::string msg = bubble_last_error();
            bubble_destroy(sim);
            die(msg, 1);
        }
        std::printf("checkpoint %s (step %llu)\n", a.save_checkpoint.c_str(),
                    (unsigned long long)bubble_steps(sim));
    }
    if (!a.screenshot.empty()) {
        // render_to_png (src/capture.rs:19-117) of the current state
        bubble_render_settings rs;
        bubble_render_settings_with_field(a.field, &rs);
        if (bubble_render_png(sim, &rs, a.screenshot_size[0], a.screenshot_size[1], a.screenshot.c_str()) !=
            BUBBLE_OK) {
            const std::string msg = bubble_last_error();
            bubble_destroy(sim);
            die(msg, 1);
        }
        std::printf("wrote %s (%ux%u)\n", a.screenshot.c_str(), a.screenshot_size[0], a.screenshot_size[1]);
    }
    bubble_destroy(sim);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    const Args a = parse(argc, argv);
    validate(a);
    // src/main.rs:30-34: --headless or --screenshot run windowless
    if (!a.has_headless && a.screenshot.empty())
        die("the interactive window is not part of this build; run with --headless N", 2);
    const unsigned long long steps = a.has_headless ? a.headless : 0;
    unsigned long long every = a.has_report_every ? a.report_every : steps / 20;
    if (every < 1) every = 1;
    return run(a, steps, every);
}
