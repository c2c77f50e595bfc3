// Batched form: see batch.h.
#include "batch.h"

#include <cuda_runtime_api.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>

#include "launch.h"
#include "simulation.h"

namespace bubble {

namespace {

#define BATCH_CUDA(call, what)                                                  \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) {                                                \
            err = std::string(what) + ": " + cudaGetErrorString(e_);            \
            return BUBBLE_ERR_CUDA;                                             \
        }                                                                       \
    } while (0)

LatticeParams<float> params_of(const bubble_model &m, const uint32_t grid[3]) {
    const SimParamsHost h = sim_params(m, grid);
    LatticeParams<float> p{};
    p.nx = (int)h.nx;
    p.ny = (int)h.ny;
    p.nz = (int)h.nz;
    p.dx = h.dx;
    p.inv_dx = h.inv_dx;
    p.eta = h.eta;
    p.lambda = h.lambda;
    p.phi_b = h.phi_b;
    p.m2 = h.m2;
    p.delta = h.delta;
    p.wall_width = h.wall_width;
    p.p_floor = h.p_floor;
    p.e_floor = h.e_floor;
    p.z_max = h.z_max;
    p.e_ref = h.e_ref;
    return p;
}

std::mutex g_tune_mu;
std::map<std::tuple<uint32_t, uint32_t, uint32_t, int, bool>, int> g_tune_cache;

constexpr size_t kOffStatus = 64;     // counters at 0 (16 B), status at 64
constexpr size_t kOffDiag = 256;      // diag partials | ticket | result

std::string check_spec(const bubble_spec &s, int math) {
    const std::string msg = validate_model(s.model);
    if (!msg.empty()) return msg;
    if (s.precision != BUBBLE_PRECISION_SINGLE) return "a batch runs FP32 lattices (BUBBLE_PRECISION_SINGLE)";
    if (s.eos == BUBBLE_EOS_GAMMA_LAW || s.eos == BUBBLE_EOS_THERMAL) return "a batch runs the bag equation of state";
    if (s.math != math) return "all lattices of a batch share one math mode";
    for (int a = 0; a < 3; ++a)
        if (s.grid[a] < BUBBLE_MIN_GRID || s.grid[a] > BUBBLE_MAX_GRID) return "grid axis out of 8..2048";
    if ((uint64_t)s.grid[0] * s.grid[1] * s.grid[2] > BUBBLE_MAX_CELLS) return "lattice above 2^32 - 1 cells";
    if (s.nucleation < BUBBLE_NUCLEATION_SIMULTANEOUS || s.nucleation > BUBBLE_NUCLEATION_UNIFORM)
        return "unknown nucleation mode";
    return "";
}

}  // namespace

// ---------------------------------------------------------------------------
//  Autotuner
// ---------------------------------------------------------------------------
int autotune_chunk(const uint32_t grid[3], int ty, bool fast, std::string &err) {
    const auto key = std::make_tuple(grid[0], grid[1], grid[2], ty, fast);
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) return it->second;
    }
    bubble_spec spec;
    std::memset(&spec, 0, sizeof(spec));
    spec.model = default_model();
    for (int a = 0; a < 3; ++a) spec.grid[a] = grid[a];
    spec.nucleation = BUBBLE_NUCLEATION_SIMULTANEOUS;
    spec.bubbles = 0;
    spec.nucleation_duration = 1.0f;
    spec.seed = 1;
    spec.precision = BUBBLE_PRECISION_SINGLE;
    spec.math = fast ? BUBBLE_MATH_FAST : BUBBLE_MATH_STRICT;
    std::unique_ptr<Simulation> sim;
    int rc = Simulation::create(spec, sim, err);
    if (rc != BUBBLE_OK) return -1;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        err = "cudaEventCreate failed";
        return -1;
    }
    const int nz = (int)grid[2];
    std::vector<int> cand;
    for (int lz : {4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256})
        if (lz < nz) cand.push_back(lz);
    cand.push_back(nz);
    int best = cand.front();
    float best_ms = 1e30f;
    // The quiescent initial state is an exact fixed point of the scheme, so
    // timing steps on it does not change the lattice.
    for (int lz : cand) {
        if (sim->set_tile(TileShape{tile_x_for(ty), ty, lz}, err) != BUBBLE_OK) continue;
        if (sim->record_steps(1, err) != BUBBLE_OK) break;
        cudaEventRecord(e0, sim->stream());
        if (sim->record_steps(3, err) != BUBBLE_OK) break;
        cudaEventRecord(e1, sim->stream());
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
            best_ms = ms;
            best = lz;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = best;
    return best;
}

// ---------------------------------------------------------------------------
//  Batch
// ---------------------------------------------------------------------------
int Batch::setup(int math, const bubble_batch_options *opt, std::string &err) {
    bubble_batch_options o;
    o.tile_y = 16;
    o.autotune = 1;
    o.use_graph = 1;
    o.max_grid = 0;
    if (opt) o = *opt;
    math_ = math;
    fast_ = math == BUBBLE_MATH_FAST;
    if (math != BUBBLE_MATH_FAST && math != BUBBLE_MATH_STRICT) {
        err = "unknown math mode";
        return BUBBLE_ERR_INVALID;
    }
    if (o.tile_y != 16 && !(fast_ && o.tile_y == 8)) {
        err = "batch tile_y must be 16 (16 x 16 tiles; or 8, 32 x 8 tiles, in the fast mode)";
        return BUBBLE_ERR_INVALID;
    }
    ty_ = o.tile_y;
    use_graph_ = o.use_graph != 0;
    autotuned_ = false;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        err = "no CUDA device is available (this library has no CPU path)";
        return BUBBLE_ERR_CUDA;
    }
    BATCH_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    const size_t pb = (launch::diag_partials_bytes() + 255) & ~(size_t)255;
    const size_t scratch = kOffDiag + pb + 256 + 256;
    BATCH_CUDA(cudaMalloc(&d_scratch_, scratch), "cudaMalloc");
    BATCH_CUDA(cudaMemsetAsync(d_scratch_, 0, scratch, stream_), "cudaMemset");
    d_counters_ = static_cast<unsigned int *>(d_scratch_);
    d_status_ = reinterpret_cast<int *>(static_cast<char *>(d_scratch_) + kOffStatus);
    BATCH_CUDA(cudaMallocHost(reinterpret_cast<void **>(&h_result_), sizeof(DiagResult)), "cudaMallocHost");
    device_bytes_ += scratch;
    int maxg = launch::batch_max_grid(fast_, ty_);
    if (maxg <= 0) {
        err = "the batch kernel cannot be resident on this device";
        return BUBBLE_ERR_CUDA;
    }
    if (o.max_grid > 0 && o.max_grid < maxg) maxg = o.max_grid;
    max_grid_ = maxg;
    return BUBBLE_OK;
}

int Batch::create(const bubble_spec *specs, uint32_t n, const bubble_batch_options *opt,
                  std::unique_ptr<Batch> &out, std::string &err) {
    if (n == 0) {
        err = "a batch needs at least one lattice";
        return BUBBLE_ERR_INVALID;
    }
    for (uint32_t k = 0; k < n; ++k) {
        const std::string msg = check_spec(specs[k], specs[0].math);
        if (!msg.empty()) {
            err = "lattice " + std::to_string(k) + ": " + msg;
            return BUBBLE_ERR_INVALID;
        }
    }
    // admission: the whole batch against free memory (src/gpu/vram.rs:52-69)
    uint64_t need = 0;
    for (uint32_t k = 0; k < n; ++k) need += bubble_lattice_bytes(specs[k].grid);
    size_t free_b = 0, total_b = 0;
    BATCH_CUDA(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    if ((double)need > 0.85 * (double)free_b) {
        err = "the batch needs " + std::to_string(need) + " bytes, above 85% of the " + std::to_string(free_b) +
              " bytes free";
        return BUBBLE_ERR_MEMORY;
    }
    std::unique_ptr<Batch> b(new Batch());
    int rc = b->setup(specs[0].math, opt, err);
    if (rc != BUBBLE_OK) return rc;
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t idx = 0;
        rc = b->add(specs[k], &idx, err);
        if (rc != BUBBLE_OK) return rc;
    }
    b->plan_items();
    if (!opt || opt->autotune) {
        rc = b->autotune(err);
        if (rc != BUBBLE_OK) return rc;
    }
    BATCH_CUDA(cudaStreamSynchronize(b->stream_), "cudaStreamSynchronize");
    out = std::move(b);
    return BUBBLE_OK;
}

int Batch::create_empty(int math, const bubble_batch_options *opt, std::unique_ptr<Batch> &out,
                        std::string &err) {
    std::unique_ptr<Batch> b(new Batch());
    const int rc = b->setup(math, opt, err);
    if (rc != BUBBLE_OK) return rc;
    out = std::move(b);
    return BUBBLE_OK;
}

Batch::~Batch() {
    if (stream_) cudaStreamSynchronize(stream_);
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    for (auto &L : lats_)
        if (L.state) cudaFree(L.state);
    if (d_lat_) cudaFree(d_lat_);
    if (h_lat_) cudaFreeHost(h_lat_);
    if (d_scratch_) cudaFree(d_scratch_);
    if (h_result_) cudaFreeHost(h_result_);
    if (stream_) cudaStreamDestroy(stream_);
}

uint32_t Batch::active_count() const {
    uint32_t n = 0;
    for (const auto &L : lats_) n += L.state != nullptr;
    return n;
}

int Batch::allocate(Lat &L, std::string &err) {
    auto round_up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t fb = round_up(L.cells * 8), ub = round_up(L.cells * 16);
    const size_t slot = fb + ub;
    cudaError_t e = cudaMalloc(&L.state, 3 * slot);
    if (e != cudaSuccess) {
        cudaGetLastError();
        L.state = nullptr;
        err = std::string("device allocation of a batch lattice failed: ") + cudaGetErrorString(e);
        return BUBBLE_ERR_MEMORY;
    }
    L.bytes = 3 * slot;
    device_bytes_ += L.bytes;
    L.tma_ok = true;
    for (int k = 0; k < 3; ++k) {
        L.field[k] = static_cast<char *>(L.state) + k * slot;
        L.fluid[k] = static_cast<char *>(L.state) + k * slot + fb;
        L.tma_ok = L.tma_ok && encode_stage_maps(&L.maps[k], L.field[k], L.fluid[k], (int)L.grid[0],
                                                 (int)L.grid[1], (int)L.grid[2], tile_x_for(ty_), ty_, 4);
    }
    BATCH_CUDA(launch::init_f32((V2<float> *)L.field[0], (V4<float> *)L.fluid[0], L.cells, L.P.e_ref, stream_),
               "init kernel");
    ++launches_;
    return BUBBLE_OK;
}

int Batch::add(const bubble_spec &spec, uint32_t *index, std::string &err) {
    const std::string msg = check_spec(spec, math_);
    if (!msg.empty()) {
        err = msg;
        return BUBBLE_ERR_INVALID;
    }
    Lat L;
    L.spec = spec;
    std::memcpy(L.grid, spec.grid, sizeof(L.grid));
    L.cells = (uint64_t)L.grid[0] * L.grid[1] * L.grid[2];
    L.P = params_of(spec.model, L.grid);
    const Derived d = derive(spec.model);
    L.dt = d.dt;
    L.schedule = make_schedule(spec.nucleation, spec.bubbles, d.seed_radius, L.grid, spec.nucleation_duration,
                               spec.seed);
    {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const long tx = tile_x_for(ty_);
        const long tiles = (long)((L.grid[0] + tx - 1) / tx) * (long)((L.grid[1] + ty_ - 1) / ty_);
        L.solo = tiles * (((long)L.grid[2] + 31) / 32) >= 2L * std::max(sms, 1);
        if (L.solo) {
            L.lz = default_chunk(L.grid, ty_, true);
        } else {
            // equal chunks no longer than the cap
            const int nz = (int)L.grid[2];
            const int pieces = (nz + lz_cap_ - 1) / lz_cap_;
            L.lz = (nz + pieces - 1) / pieces;
        }
    }
    const int rc = allocate(L, err);
    if (rc != BUBBLE_OK) return rc;
    lats_.push_back(std::move(L));
    *index = (uint32_t)(lats_.size() - 1);
    dirty_ = true;
    return BUBBLE_OK;
}

int Batch::remove(uint32_t k, std::string &err) {
    if (!active(k)) {
        err = "no active lattice at this index";
        return BUBBLE_ERR_INVALID;
    }
    BATCH_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    Lat &L = lats_[k];
    BATCH_CUDA(cudaFree(L.state), "cudaFree");
    device_bytes_ -= L.bytes;
    L.state = nullptr;
    for (int s = 0; s < 3; ++s) L.field[s] = L.fluid[s] = nullptr;
    L.schedule.clear();
    L.schedule.shrink_to_fit();
    dirty_ = true;
    return BUBBLE_OK;
}

// Items of a stage for the active lattices (largest first) and the grid.
void Batch::plan_items() {
    item_order_.clear();
    for (uint32_t k = 0; k < lats_.size(); ++k)
        if (lats_[k].state && !lats_[k].solo) item_order_.push_back(k);
    std::stable_sort(item_order_.begin(), item_order_.end(),
                     [&](uint32_t a, uint32_t c) { return lats_[a].cells > lats_[c].cells; });
    const int tx = tile_x_for(ty_);
    auto count_items = [&]() {
        int n = 0;
        for (uint32_t k : item_order_) {
            const Lat &L = lats_[k];
            const int tiles = (int)((L.grid[0] + tx - 1) / tx) * (int)((L.grid[1] + ty_ - 1) / ty_);
            n += tiles * (int)((L.grid[2] + L.lz - 1) / L.lz);
        }
        return n;
    };
    if (fill_) {
        // Equal chunks no longer than the cap, the cap chosen among the
        // configured one and shorter ones by a cost per stage round: the
        // item-planes (each chunk's planes plus 2 warm-up planes) spread
        // over the persistent grid, plus the longest item (the round's
        // tail).  Any chunking gives the same bits.
        auto apply = [&](int cap) {
            for (uint32_t k : item_order_) {
                Lat &L = lats_[k];
                const int nz = (int)L.grid[2];
                const int pieces = (nz + cap - 1) / cap;
                L.lz = (nz + pieces - 1) / pieces;
            }
        };
        double best = 1e300;
        int best_cap = lz_cap_;
        for (int cap : {lz_cap_, 48, 32, 24, 16, 12, 8, 6, 4}) {
            if (cap > lz_cap_) continue;
            apply(cap);
            double planes = 0.0;
            int longest = 0;
            for (uint32_t k : item_order_) {
                const Lat &L = lats_[k];
                const long tiles = (long)((L.grid[0] + tx - 1) / tx) * (long)((L.grid[1] + ty_ - 1) / ty_);
                const long chunks = ((long)L.grid[2] + L.lz - 1) / L.lz;
                planes += (double)tiles * (double)(L.grid[2] + 2 * chunks);
                longest = std::max(longest, L.lz + 2);
            }
            const double cost = planes / (double)std::max(1, max_grid_) + (double)longest;
            if (cost < best * (1.0 - 1e-9)) {
                best = cost;
                best_cap = cap;
            }
        }
        apply(best_cap);
    }
    n_items_ = count_items();
    grid_ = std::max(1, std::min(max_grid_, n_items_));
    dirty_ = false;
}

int Batch::ensure_capacity(size_t n, std::string &err) {
    if (n <= capacity_) return BUBBLE_OK;
    size_t cap = std::max<size_t>(n, capacity_ * 2);
    cap = std::max<size_t>(cap, 16);
    BATCH_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
    graph_ok_ = false;  // the captured memcpy referenced the old buffers
    if (d_lat_) cudaFree(d_lat_);
    if (h_lat_) cudaFreeHost(h_lat_);
    d_lat_ = nullptr;
    h_lat_ = nullptr;
    BATCH_CUDA(cudaMalloc(reinterpret_cast<void **>(&d_lat_), sizeof(BatchLattice) * cap), "cudaMalloc");
    BATCH_CUDA(cudaMallocHost(reinterpret_cast<void **>(&h_lat_), sizeof(BatchLattice) * cap), "cudaMallocHost");
    device_bytes_ += sizeof(BatchLattice) * (cap - capacity_);
    capacity_ = cap;
    return BUBBLE_OK;
}

// Chooses the z chunks of the batch by timing the batch itself.  The
// candidates are each size's single-lattice optimum (tuned for filling the
// GPU with one lattice) and caps (whole columns, then 96, 64, 48, 32 and 24
// planes, each column cut into equal chunks no longer than the cap), which
// trade the 5-plane prologue of every chunk against the tail of each
// stage's round once the batch fills the GPU.  The lattices are still in
// their quiescent initial state, an exact fixed point, so the timing steps
// change nothing.  Solo lattices keep their plain-path chunk.
int Batch::autotune(std::string &err) {
    std::vector<std::vector<int>> cands;
    std::vector<int> single;
    for (auto &L : lats_) {
        if (L.solo) {  // runs alone with the plain path's chunk
            single.push_back(L.lz);
            continue;
        }
        const int lz = autotune_chunk(L.grid, ty_, fast_, err);
        if (lz <= 0) return BUBBLE_ERR_CUDA;
        single.push_back(lz);
    }
    cands.push_back(single);
    for (int cap : {1 << 30, 96, 64, 48, 32, 24}) {
        std::vector<int> c;
        for (auto &L : lats_) {
            const int nz = (int)L.grid[2];
            const int pieces = (nz + cap - 1) / cap;
            c.push_back(L.solo ? L.lz : (nz + pieces - 1) / pieces);
        }
        if (std::find(cands.begin(), cands.end(), c) == cands.end()) cands.push_back(c);
    }
    cudaEvent_t e0, e1;
    BATCH_CUDA(cudaEventCreate(&e0), "cudaEventCreate");
    BATCH_CUDA(cudaEventCreate(&e1), "cudaEventCreate");
    const bool graph = use_graph_;
    use_graph_ = false;
    float best_ms = 1e30f;
    size_t best = 0;
    for (size_t c = 0; c < cands.size(); ++c) {
        for (size_t k = 0; k < lats_.size(); ++k) lats_[k].lz = cands[c][k];
        plan_items();
        int rc = launch_chunk(1, err);
        if (rc != BUBBLE_OK) return rc;
        BATCH_CUDA(cudaEventRecord(e0, stream_), "cudaEventRecord");
        rc = launch_chunk(2, err);
        if (rc != BUBBLE_OK) return rc;
        BATCH_CUDA(cudaEventRecord(e1, stream_), "cudaEventRecord");
        BATCH_CUDA(cudaEventSynchronize(e1), "cudaEventSynchronize");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    use_graph_ = graph;
    for (size_t k = 0; k < lats_.size(); ++k) lats_[k].lz = cands[best][k];
    plan_items();
    autotuned_ = true;
    return check_status(err);
}

// record_nucleation (src/gpu/sim.rs:843-879) for one lattice.
int Batch::nucleate_due(Lat &L, std::string &err) {
    V4<float> batch[BUBBLE_MAX_BATCH];
    int count = 0;
    while (L.next_event < L.schedule.size() && L.schedule[L.next_event].time <= L.time &&
           count < (int)BUBBLE_MAX_BATCH) {
        const bubble_event &e = L.schedule[L.next_event];
        batch[count++] = V4<float>{e.pos[0], e.pos[1], e.pos[2], e.radius};
        ++L.next_event;
    }
    if (count == 0) return BUBBLE_OK;
    BATCH_CUDA(launch::nucleate_f32((V2<float> *)L.field[L.cur], batch, count, L.P, stream_), "nucleate kernel");
    launches_ += (count + 127) / 128;
    return BUBBLE_OK;
}

// Steps the lattice can take before a nucleation check would find an event
// due: the smallest j >= 1 with the time after j steps >= the next event's
// time (f32 accumulation, as src/gpu/sim.rs:914).
uint64_t Batch::steps_until_event(const Lat &L, uint64_t cap) const {
    if (L.next_event >= L.schedule.size()) return cap;
    const float te = L.schedule[L.next_event].time;
    float t = L.time;
    for (uint64_t j = 1; j <= cap; ++j) {
        t += L.dt;
        if (t >= te) return j;
    }
    return cap;
}

int Batch::launch_chunk(uint64_t k, std::string &err) {
    if (item_order_.empty() || k == 0) return BUBBLE_OK;
    int rc = ensure_capacity(item_order_.size(), err);
    if (rc != BUBBLE_OK) return rc;
    // the previous launch has consumed the pinned descriptors
    BATCH_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    int begin = 0;
    for (size_t q = 0; q < item_order_.size(); ++q) {
        const Lat &L = lats_[item_order_[q]];
        BatchLattice &D = h_lat_[q];
        std::memset(&D, 0, sizeof(D));
        for (int s = 0; s < 3; ++s) {
            D.maps[s] = L.maps[s];
            D.field[s] = (V2<float> *)L.field[s];
            D.fluid[s] = (V4<float> *)L.fluid[s];
        }
        D.P = L.P;
        D.dt = L.dt;
        D.lz = L.lz;
        D.tiles_xy = (int)((L.grid[0] + tile_x_for(ty_) - 1) / tile_x_for(ty_)) * (int)((L.grid[1] + ty_ - 1) / ty_);
        D.chunks = (int)((L.grid[2] + L.lz - 1) / L.lz);
        D.item_begin = begin;
        D.cur0 = (int)L.cur;
        D.tma_ok = L.tma_ok ? 1 : 0;
        begin += D.tiles_xy * D.chunks;
    }
    const size_t lat_bytes = sizeof(BatchLattice) * item_order_.size();
    const int n_lat = (int)item_order_.size();
    auto enqueue = [&]() -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(d_lat_, h_lat_, lat_bytes, cudaMemcpyHostToDevice, stream_);
        if (e == cudaSuccess) e = cudaMemsetAsync(d_counters_, 0, 16, stream_);
        if (e == cudaSuccess)
            e = launch::batch_launch(fast_, ty_, d_lat_, n_lat, n_items_, (int)k, d_counters_, d_status_, grid_,
                                     test_barrier_shift_ ? 1u : 0u, test_barrier_shift_ ? test_barrier_shift_ : 32,
                                     stream_);
        return e;
    };
    if (test_barrier_shift_) {
        // test hook: one direct launch whose grid barrier no arrival releases
        const cudaError_t e = enqueue();
        test_barrier_shift_ = 0;
        BATCH_CUDA(e, "batch launch");
        ++launches_;
        return BUBBLE_OK;
    }
    if (use_graph_) {
        const auto key = std::make_tuple(k, n_lat, n_items_, grid_);
        if (!graph_ok_ || graph_key_ != key) {
            if (exec_) cudaGraphExecDestroy(exec_);
            if (graph_) cudaGraphDestroy(graph_);
            exec_ = nullptr;
            graph_ = nullptr;
            graph_ok_ = false;
            cudaError_t e = cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal);
            cudaError_t e2 = e == cudaSuccess ? enqueue() : e;
            cudaGraph_t g = nullptr;
            cudaError_t e3 = e == cudaSuccess ? cudaStreamEndCapture(stream_, &g) : e;
            if (e2 == cudaSuccess && e3 == cudaSuccess && g) {
                graph_ = g;
                if (cudaGraphInstantiate(&exec_, graph_, 0) == cudaSuccess) {
                    graph_ok_ = true;
                    graph_key_ = key;
                }
            } else if (g) {
                cudaGraphDestroy(g);
            }
            if (!graph_ok_) {
                cudaGetLastError();
                use_graph_ = false;  // this device/driver cannot capture it: launch directly
            }
        }
        if (graph_ok_) {
            BATCH_CUDA(cudaGraphLaunch(exec_, stream_), "cudaGraphLaunch");
            ++launches_;
            return BUBBLE_OK;
        }
    }
    BATCH_CUDA(enqueue(), "batch launch");
    ++launches_;
    return BUBBLE_OK;
}

int Batch::advance(uint64_t steps, std::string &err) {
    if (dirty_) plan_items();
    uint64_t done = 0;
    while (done < steps) {
        for (auto &L : lats_) {
            if (!L.state) continue;
            const int rc = nucleate_due(L, err);
            if (rc != BUBBLE_OK) return rc;
        }
        uint64_t k = steps - done;
        for (const auto &L : lats_)
            if (L.state) k = std::min(k, steps_until_event(L, k));
        // the kernel numbers the grabs of a launch's rounds in 32 bits
        k = std::min<uint64_t>(
            k, std::max<uint64_t>(1, 0x7fffffffull / (3ull * (uint64_t)(std::max(n_items_, 1) + grid_))));
        int rc = launch_chunk(k, err);
        if (rc != BUBBLE_OK) return rc;
        for (auto &L : lats_) {
            if (!L.state || !L.solo) continue;
            rc = launch_solo(L, k, err);
            if (rc != BUBBLE_OK) return rc;
        }
        for (auto &L : lats_) {
            if (!L.state) continue;
            L.cur = (uint32_t)((L.cur + k) % 3);
            for (uint64_t j = 0; j < k; ++j) L.time += L.dt;
            L.steps += k;
        }
        done += k;
    }
    return BUBBLE_OK;
}

// k steps of one solo lattice: three stage launches per step, the slot
// rotation of src/gpu/sim.rs:1046-1051, on the batch's stream after its
// shared launch.
int Batch::launch_solo(Lat &L, uint64_t k, std::string &err) {
    for (uint64_t j = 0; j < k; ++j) {
        const uint32_t cur = (uint32_t)((L.cur + j) % 3);
        uint32_t in[3], out[3];
        stage_slots(cur, in, out);
        for (int st = 0; st < 3; ++st) {
            StageArgs<float> A;
            A.field_n = (const V2<float> *)L.field[cur];
            A.fluid_n = (const V4<float> *)L.fluid[cur];
            A.field_in = (const V2<float> *)L.field[in[st]];
            A.fluid_in = (const V4<float> *)L.fluid[in[st]];
            A.field_out = (V2<float> *)L.field[out[st]];
            A.fluid_out = (V4<float> *)L.fluid[out[st]];
            A.a0 = kRK3[st][0];
            A.a1 = kRK3[st][1];
            A.dt = L.dt;
            A.stage = st;
            const TileShape tile{tile_x_for(ty_), ty_, L.lz};
            const int tma = L.tma_ok ? 1 : 0;
            const cudaError_t e =
                fast_ ? launch::stage_f32_fast(A, L.P, tile, 0, L.maps[in[st]], tma, d_status_, stream_)
                      : launch::stage_f32_strict(A, L.P, tile, 0, L.maps[in[st]], tma, d_status_, stream_);
            BATCH_CUDA(e, "stage kernel of a solo lattice");
            ++launches_;
        }
    }
    return BUBBLE_OK;
}

int Batch::check_status(std::string &err) {
    int st[16] = {0};
    BATCH_CUDA(cudaMemcpyAsync(st, d_status_, sizeof(st), cudaMemcpyDeviceToHost, stream_), "status readback");
    BATCH_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    if (st[0] != 0) {
        BATCH_CUDA(cudaMemsetAsync(d_status_, 0, sizeof(st), stream_), "cudaMemset");
        err = "a batch launch gave up on a bounded wait (status " + std::to_string(st[0]) + ")";
        if (st[8])
            err += "; stage wait gave up in item " + std::to_string(st[9]) + " (lattice " + std::to_string(st[10]) +
                   ", round " + std::to_string(st[11]) + ", local item " + std::to_string(st[12]) + ")";
        return BUBBLE_ERR_TIMEOUT;
    }
    return BUBBLE_OK;
}

int Batch::diagnostics(uint32_t k, bubble_diag *out, std::string &err) {
    if (!active(k)) {
        err = "no active lattice at this index";
        return BUBBLE_ERR_INVALID;
    }
    const Lat &L = lats_[k];
    const size_t pb = (launch::diag_partials_bytes() + 255) & ~(size_t)255;
    char *base = static_cast<char *>(d_scratch_) + kOffDiag;
    unsigned int *ticket = reinterpret_cast<unsigned int *>(base + pb);
    DiagResult *res = reinterpret_cast<DiagResult *>(base + pb + 256);
    BATCH_CUDA(launch::diag_f32((const V2<float> *)L.field[L.cur], (const V4<float> *)L.fluid[L.cur], L.P, false,
                                base, ticket, res, stream_),
               "diagnostics kernel");
    BATCH_CUDA(cudaMemcpyAsync(h_result_, res, sizeof(DiagResult), cudaMemcpyDeviceToHost, stream_),
               "diagnostics readback");
    const int rc = check_status(err);
    if (rc != BUBBLE_OK) return rc;
    const DiagResult &r = *h_result_;
    const float inv_n = 1.0f / (float)L.cells;
    bubble_diag d{};
    d.sum_energy = r.sums[0];
    d.sum_broken = r.sums[1];
    d.sum_kinetic = r.sums[2];
    d.sum_fluid_energy = r.sums[3];
    d.mean_energy = (float)r.sums[0] * inv_n;
    d.broken_fraction = (float)r.sums[1] * inv_n;
    d.mean_kinetic = (float)r.sums[2] * inv_n;
    d.mean_fluid_energy = (float)r.sums[3] * inv_n;
    std::memcpy(&d.max_velocity, &r.max_v_bits, sizeof(float));
    d.kinetic_fraction = std::fabs(d.mean_energy) < 1e-20f ? 0.0f : d.mean_kinetic / d.mean_energy;
    d.mean_energy_f64 = r.sums[0] / (double)L.cells;
    d.mean_kinetic_f64 = r.sums[2] / (double)L.cells;
    d.cells = L.cells;
    *out = d;
    if (r.nonfinite || !std::isfinite(d.mean_energy) || !std::isfinite(d.max_velocity)) {
        err = "lattice " + std::to_string(k) + " blew up (non-finite diagnostics)";
        return BUBBLE_ERR_NONFINITE;
    }
    return BUBBLE_OK;
}

int Batch::copy_state(uint32_t k, float *field, float *fluid, std::string &err) {
    if (!active(k)) {
        err = "no active lattice at this index";
        return BUBBLE_ERR_INVALID;
    }
    const Lat &L = lats_[k];
    BATCH_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    if (field) BATCH_CUDA(cudaMemcpy(field, L.field[L.cur], L.cells * 8, cudaMemcpyDeviceToHost), "state readback");
    if (fluid) BATCH_CUDA(cudaMemcpy(fluid, L.fluid[L.cur], L.cells * 16, cudaMemcpyDeviceToHost), "state readback");
    return check_status(err);
}

int Batch::load_state(uint32_t k, const float *field, const float *fluid, std::string &err) {
    if (!active(k)) {
        err = "no active lattice at this index";
        return BUBBLE_ERR_INVALID;
    }
    const Lat &L = lats_[k];
    BATCH_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    if (field) BATCH_CUDA(cudaMemcpy(L.field[L.cur], field, L.cells * 8, cudaMemcpyHostToDevice), "state upload");
    if (fluid) BATCH_CUDA(cudaMemcpy(L.fluid[L.cur], fluid, L.cells * 16, cudaMemcpyHostToDevice), "state upload");
    return BUBBLE_OK;
}

void Batch::info(bubble_batch_info *out) const {
    std::memset(out, 0, sizeof(*out));
    out->lattices = active_count();
    out->grid = (uint32_t)grid_;
    out->items = (uint32_t)n_items_;
    out->tile_y = ty_;
    out->graph = graph_ok_ ? 1 : 0;
    out->autotuned = autotuned_ ? 1 : 0;
    for (const auto &L : lats_)
        if (L.state) out->cells += L.cells;
    out->launches = launches_;
    out->device_bytes = device_bytes_;
}

}  // namespace bubble
