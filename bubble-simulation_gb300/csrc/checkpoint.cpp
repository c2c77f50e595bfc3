// Raw-state checkpoint and resume of one simulation.
//
// The reference keeps no checkpoint: its state lives only in device buffers
// (src/gpu/sim.rs:180-245).  A checkpoint here holds what a bit-exact
// continuation needs: the spec (model, grid, nucleation settings,
// precision, arithmetic mode), the clock (f32 time, step count), the
// schedule and how far it has been consumed, and the current slot's field
// and fluid arrays.  The other two RK slots are scratch at a step boundary,
// so the state is restored into slot 0 and stepping continues identically.
//
// File layout (little-endian, as written by the host):
//   char[8]  "BUBCKPT1"
//   u32      header bytes (sizeof(Header))
//   Header   spec, time, steps, next_event, n_events, cells, bytes per cell
//   bubble_event[n_events]
//   field[cells], fluid[cells]   (FP32 or FP64 as the precision says)
//   u32      CRC-32 of every byte before it
#include <cuda_runtime_api.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "physics.h"
#include "simulation.h"

#include "../../include/bubble_checkpoint.h"
#include "sim_handle.h"

namespace bubble {

namespace {

#define CKPT_CUDA(call, what)                                                  \
    do {                                                                       \
        const cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) {                                               \
            err = std::string(what) + ": " + cudaGetErrorString(e_);           \
            return BUBBLE_ERR_CUDA;                                            \
        }                                                                      \
    } while (0)

constexpr char kMagic[8] = {'B', 'U', 'B', 'C', 'K', 'P', 'T', '1'};

struct Header {
    bubble_spec spec;
    float time;
    uint32_t field_bytes_per_cell;
    uint64_t steps;
    uint64_t next_event;
    uint64_t n_events;
    uint64_t cells;
    uint32_t fluid_bytes_per_cell;
    uint32_t reserved;
};

// CRC-32 (reflected polynomial 0xEDB88320) lookup table, built at compile time
// so concurrent saves and loads share it without any initialisation race.
struct Crc32Table {
    uint32_t t[256];
    constexpr Crc32Table() : t() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
    }
};
constexpr Crc32Table kCrc32Table{};

uint32_t crc32_of(const unsigned char *p, size_t n, uint32_t crc = 0xFFFFFFFFu) {
    for (size_t i = 0; i < n; ++i) crc = kCrc32Table.t[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return crc;
}

// Reads and checks a whole checkpoint file: magic, sizes, CRC.
int read_file(const std::string &path, std::vector<unsigned char> &buf, Header &h, std::string &err) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err = "cannot open " + path;
        return BUBBLE_ERR_INVALID;
    }
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (size < 0) {
        std::fclose(f);
        err = "cannot read " + path;
        return BUBBLE_ERR_INVALID;
    }
    buf.resize((size_t)size);
    const size_t got = std::fread(buf.data(), 1, buf.size(), f);
    std::fclose(f);
    const size_t fixed = sizeof(kMagic) + 4 + sizeof(Header) + 4;
    if (got != buf.size() || buf.size() < fixed || std::memcmp(buf.data(), kMagic, sizeof(kMagic)) != 0) {
        err = path + " is not a bubble checkpoint";
        return BUBBLE_ERR_INVALID;
    }
    uint32_t hb;
    std::memcpy(&hb, buf.data() + 8, 4);
    if (hb != sizeof(Header)) {
        err = path + ": unsupported checkpoint header";
        return BUBBLE_ERR_INVALID;
    }
    std::memcpy(&h, buf.data() + 12, sizeof(Header));
    const bool f64 = h.spec.precision == BUBBLE_PRECISION_DOUBLE;
    const uint64_t want_field = f64 ? 16 : 8, want_fluid = f64 ? 32 : 16;
    const uint64_t cells = (uint64_t)h.spec.grid[0] * h.spec.grid[1] * h.spec.grid[2];
    if (h.field_bytes_per_cell != want_field || h.fluid_bytes_per_cell != want_fluid || h.cells != cells ||
        h.next_event > h.n_events || h.n_events > (uint64_t)1 << 32) {
        err = path + ": inconsistent checkpoint header";
        return BUBBLE_ERR_INVALID;
    }
    const uint64_t body = (uint64_t)h.n_events * sizeof(bubble_event) + cells * (want_field + want_fluid);
    if ((uint64_t)buf.size() != fixed + body) {
        err = path + ": truncated or oversized checkpoint";
        return BUBBLE_ERR_INVALID;
    }
    uint32_t crc;
    std::memcpy(&crc, buf.data() + buf.size() - 4, 4);
    if ((crc32_of(buf.data(), buf.size() - 4) ^ 0xFFFFFFFFu) != crc) {
        err = path + ": checksum mismatch";
        return BUBBLE_ERR_INVALID;
    }
    return BUBBLE_OK;
}

}  // namespace

int Simulation::save_checkpoint(const std::string &path, std::string &err) {
    if (!state_) {
        err = "the simulation holds no lattice";
        return BUBBLE_ERR_INVALID;
    }
    Header h;
    std::memset(&h, 0, sizeof(h));
    h.spec = spec_;
    h.time = time_;
    h.steps = steps_;
    h.next_event = next_event_;
    h.n_events = schedule_.size();
    h.cells = n_cells_;
    h.field_bytes_per_cell = (uint32_t)elem_field();
    h.fluid_bytes_per_cell = (uint32_t)elem_fluid();
    std::vector<unsigned char> buf;
    const size_t state_bytes = (size_t)n_cells_ * (elem_field() + elem_fluid());
    buf.reserve(sizeof(kMagic) + 4 + sizeof(h) + schedule_.size() * sizeof(bubble_event) + state_bytes + 4);
    buf.insert(buf.end(), kMagic, kMagic + sizeof(kMagic));
    const uint32_t hb = sizeof(Header);
    buf.insert(buf.end(), (const unsigned char *)&hb, (const unsigned char *)&hb + 4);
    buf.insert(buf.end(), (const unsigned char *)&h, (const unsigned char *)&h + sizeof(h));
    if (!schedule_.empty())
        buf.insert(buf.end(), (const unsigned char *)schedule_.data(),
                   (const unsigned char *)(schedule_.data() + schedule_.size()));
    const size_t at = buf.size();
    buf.resize(at + state_bytes);
    const int rc = copy_state(buf.data() + at, buf.data() + at + (size_t)n_cells_ * elem_field(), is_f64(), err);
    if (rc != BUBBLE_OK) return rc;
    const uint32_t crc = crc32_of(buf.data(), buf.size()) ^ 0xFFFFFFFFu;
    buf.insert(buf.end(), (const unsigned char *)&crc, (const unsigned char *)&crc + 4);
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        err = "cannot create " + path;
        return BUBBLE_ERR_INVALID;
    }
    const size_t wrote = std::fwrite(buf.data(), 1, buf.size(), f);
    if (std::fclose(f) != 0 || wrote != buf.size()) {
        err = "failed to write " + path;
        return BUBBLE_ERR_INVALID;
    }
    return BUBBLE_OK;
}

int Simulation::checkpoint_spec(const std::string &path, bubble_spec &spec, std::string &err) {
    std::vector<unsigned char> buf;
    Header h;
    const int rc = read_file(path, buf, h, err);
    if (rc != BUBBLE_OK) return rc;
    spec = h.spec;
    return BUBBLE_OK;
}

int Simulation::restore_checkpoint(const std::string &path, std::string &err) {
    std::vector<unsigned char> buf;
    Header h;
    int rc = read_file(path, buf, h, err);
    if (rc != BUBBLE_OK) return rc;
    if (h.spec.precision == BUBBLE_PRECISION_DOUBLE) {
        if (!is_f64()) {
            err = "the checkpoint holds FP64 state and this simulation FP32";
            return BUBBLE_ERR_INVALID;
        }
    } else if (is_f64()) {
        err = "the checkpoint holds FP32 state and this simulation FP64";
        return BUBBLE_ERR_INVALID;
    }
    if ((h.spec.precision == BUBBLE_PRECISION_PERTURBATION) != (spec_.precision == BUBBLE_PRECISION_PERTURBATION)) {
        err = "the perturbation form stores E - e_ref: its checkpoints restore only into the perturbation form";
        return BUBBLE_ERR_INVALID;
    }
    const std::string msg = validate_model(h.spec.model);
    if (!msg.empty()) {
        err = path + ": " + msg;
        return BUBBLE_ERR_INVALID;
    }
    {
        bubble_spec chk = h.spec;
        chk.precision = spec_.precision;
        const std::string emsg = validate_eos(chk);
        if (!emsg.empty()) {
            err = path + ": " + emsg;
            return BUBBLE_ERR_INVALID;
        }
    }
    if (std::memcmp(h.spec.grid, grid_, sizeof(grid_)) != 0) {
        rc = resize(h.spec.grid, err);
        if (rc != BUBBLE_OK) return rc;
    }
    CKPT_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    // The arithmetic (single or mixed FP32, fast or strict) stays this
    // simulation's; everything else comes from the checkpoint.  The default
    // tile of a perturbation or strict simulation is already a legal one.
    const int precision = spec_.precision, math = spec_.math;
    spec_ = h.spec;
    spec_.precision = precision;
    spec_.math = math;
    const unsigned char *p = buf.data() + 12 + sizeof(Header);
    schedule_.assign((const bubble_event *)p, (const bubble_event *)p + h.n_events);
    p += h.n_events * sizeof(bubble_event);
    next_event_ = (size_t)h.next_event;
    time_ = h.time;
    steps_ = h.steps;
    cur_ = 0;
    return load_state(p, p + (size_t)n_cells_ * elem_field(), is_f64(), err);
}

}  // namespace bubble

namespace {
int fail(int code, const std::string &msg) {
    bubble::set_last_error(msg);
    return code;
}
}  // namespace

extern "C" {

int bubble_checkpoint_save(bubble_sim *sim, const char *path) {
    if (!sim || !path) return fail(BUBBLE_ERR_INVALID, "sim and path must be non-NULL");
    std::string err;
    const int rc = sim->impl->save_checkpoint(path, err);
    return rc == BUBBLE_OK ? rc : fail(rc, err);
}

int bubble_checkpoint_restore(bubble_sim *sim, const char *path) {
    if (!sim || !path) return fail(BUBBLE_ERR_INVALID, "sim and path must be non-NULL");
    std::string err;
    const int rc = sim->impl->restore_checkpoint(path, err);
    return rc == BUBBLE_OK ? rc : fail(rc, err);
}

int bubble_checkpoint_spec(const char *path, bubble_spec *out) {
    if (!path || !out) return fail(BUBBLE_ERR_INVALID, "path and out must be non-NULL");
    std::string err;
    const int rc = bubble::Simulation::checkpoint_spec(path, *out, err);
    return rc == BUBBLE_OK ? rc : fail(rc, err);
}

int bubble_checkpoint_open(const char *path, bubble_sim **out) {
    if (!path || !out) return fail(BUBBLE_ERR_INVALID, "path and out must be non-NULL");
    *out = nullptr;
    bubble_spec spec;
    int rc = bubble_checkpoint_spec(path, &spec);
    if (rc != BUBBLE_OK) return rc;
    bubble_sim *sim = nullptr;
    rc = bubble_create(&spec, &sim);
    if (rc != BUBBLE_OK) return rc;
    rc = bubble_checkpoint_restore(sim, path);
    if (rc != BUBBLE_OK) {
        bubble_destroy(sim);
        return rc;
    }
    *out = sim;
    return BUBBLE_OK;
}

}  // extern "C"
