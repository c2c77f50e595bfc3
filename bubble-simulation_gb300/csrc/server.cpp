// Serving form: include/bubble_server.h.  A FIFO of requests, admission
// against free device memory, and continuous batching over Batch.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/bubble_server.h"
#include "batch.h"
#include "physics.h"

namespace bubble {

class Server {
   public:
    static int create(const bubble_server_options &o, std::unique_ptr<Server> &out, std::string &err) {
        std::unique_ptr<Server> s(new Server());
        s->opt_ = o;
        if (s->opt_.chunk_steps == 0) s->opt_.chunk_steps = 50;
        if (s->opt_.max_active == 0) s->opt_.max_active = 64;
        if (!(s->opt_.memory_fraction > 0.0f) || s->opt_.memory_fraction > 1.0f) s->opt_.memory_fraction = 0.85f;
        bubble_batch_options bo;
        bo.tile_y = o.tile_y ? o.tile_y : 16;
        bo.autotune = 0;
        bo.use_graph = o.use_graph;
        bo.max_grid = 0;
        const int rc = Batch::create_empty(o.math, &bo, s->batch_, err);
        if (rc != BUBBLE_OK) return rc;
        s->batch_->set_chunk_planes((int)o.chunk_planes);
        s->t0_ = std::chrono::steady_clock::now();
        out = std::move(s);
        return BUBBLE_OK;
    }

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
    }

    int submit(const bubble_spec &spec, uint64_t steps, uint64_t *id, std::string &err) {
        const std::string msg = validate_model(spec.model);
        if (!msg.empty()) {
            err = msg;
            return BUBBLE_ERR_INVALID;
        }
        if (spec.precision != BUBBLE_PRECISION_SINGLE || spec.math != opt_.math) {
            err = "requests must be FP32 with the server's math mode";
            return BUBBLE_ERR_INVALID;
        }
        for (int a = 0; a < 3; ++a)
            if (spec.grid[a] < BUBBLE_MIN_GRID || spec.grid[a] > BUBBLE_MAX_GRID) {
                err = "grid axis out of 8..2048";
                return BUBBLE_ERR_INVALID;
            }
        if ((uint64_t)spec.grid[0] * spec.grid[1] * spec.grid[2] > BUBBLE_MAX_CELLS) {
            err = "lattice above 2^32 - 1 cells";
            return BUBBLE_ERR_INVALID;
        }
        Req r;
        r.id = next_id_++;
        r.spec = spec;
        r.steps = steps;
        r.submit = now();
        queue_.push_back(r);
        ++submitted_;
        if (first_submit_ < 0) first_submit_ = r.submit;
        *id = r.id;
        return BUBBLE_OK;
    }

    static uint64_t cells_of(const bubble_spec &s) { return (uint64_t)s.grid[0] * s.grid[1] * s.grid[2]; }

    // Admission: scan the queue in policy order; admit a request while a
    // resident slot is free, the resident cells stay within the budget (or
    // nothing is resident) and its lattice fits in the configured share of
    // free device memory (src/gpu/vram.rs:52-69).  A request that does not
    // fit stays queued and later, smaller ones may backfill.
    int admit(std::string &err) {
        std::vector<size_t> order(queue_.size());
        for (size_t q = 0; q < order.size(); ++q) order[q] = q;
        if (opt_.policy == BUBBLE_SERVE_SHORTEST)
            std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
                return (double)cells_of(queue_[a].spec) * queue_[a].steps <
                       (double)cells_of(queue_[b].spec) * queue_[b].steps;
            });
        const uint64_t budget = opt_.resident_cells ? opt_.resident_cells : 24ull * 1000 * 1000;
        uint64_t resident = 0;
        for (const auto &kv : active_) resident += cells_of(kv.second.req.spec);
        std::vector<bool> taken(queue_.size(), false);
        for (size_t q : order) {
            if (active_.size() >= opt_.max_active) break;
            const Req &r = queue_[q];
            const uint64_t cells = cells_of(r.spec);
            if (!active_.empty() && resident + cells > budget) continue;
            size_t free_b = 0, total_b = 0;
            if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
                cudaGetLastError();
                err = "cudaMemGetInfo failed";
                return BUBBLE_ERR_CUDA;
            }
            const uint64_t need = bubble_lattice_bytes(r.spec.grid);
            if ((double)need > (double)opt_.memory_fraction * (double)free_b) {
                if (active_.empty()) {  // can never fit: answer with an error
                    finish_error(r, BUBBLE_ERR_MEMORY);
                    taken[q] = true;
                }
                continue;
            }
            uint32_t idx = 0;
            const int rc = batch_->add(r.spec, &idx, err);
            if (rc == BUBBLE_ERR_MEMORY && !active_.empty()) continue;
            taken[q] = true;
            if (rc != BUBBLE_OK) {
                finish_error(r, rc);
                continue;
            }
            Active a;
            a.req = r;
            a.admit = now();
            a.remaining = r.steps;
            active_.emplace(idx, a);
            ++admitted_;
            resident += cells;
        }
        std::deque<Req> rest;
        for (size_t q = 0; q < queue_.size(); ++q)
            if (!taken[q]) rest.push_back(queue_[q]);
        queue_.swap(rest);
        return BUBBLE_OK;
    }

    int tick(int32_t *busy, std::string &err) {
        const int arc = admit(err);
        if (arc != BUBBLE_OK) return arc;
        if (active_.empty()) {
            *busy = queue_.empty() ? 0 : 1;
            return BUBBLE_OK;
        }
        uint64_t k = opt_.chunk_steps;
        for (const auto &kv : active_) k = std::min(k, kv.second.remaining);
        if (k > 0) {
            const int rc = batch_->advance(k, err);
            if (rc != BUBBLE_OK) return rc;
        }
        ++rounds_;
        std::vector<uint32_t> done;
        for (auto &kv : active_) {
            kv.second.remaining -= k;
            if (kv.second.remaining == 0) done.push_back(kv.first);
        }
        std::sort(done.begin(), done.end());
        for (uint32_t idx : done) {
            Active &a = active_[idx];
            bubble_server_result res;
            std::memset(&res, 0, sizeof(res));
            res.id = a.req.id;
            std::memcpy(res.grid, a.req.spec.grid, sizeof(res.grid));
            res.steps = a.req.steps;
            res.submit_s = a.req.submit;
            res.admit_s = a.admit;
            std::string derr;
            res.status = batch_->diagnostics(idx, &res.diag, derr);
            res.done_s = now();
            const int rc = batch_->remove(idx, err);
            if (rc != BUBBLE_OK) return rc;
            latencies_.push_back(res.done_s - res.submit_s);
            last_done_ = res.done_s;
            cell_updates_ += (double)a.req.spec.grid[0] * a.req.spec.grid[1] * a.req.spec.grid[2] * a.req.steps;
            results_.push_back(res);
            ++completed_;
            active_.erase(idx);
        }
        *busy = (!queue_.empty() || !active_.empty()) ? 1 : 0;
        return BUBBLE_OK;
    }

    int run_until_idle(std::string &err) {
        int32_t busy = 1;
        while (busy) {
            const int rc = tick(&busy, err);
            if (rc != BUBBLE_OK) return rc;
        }
        return BUBBLE_OK;
    }

    uint64_t poll(bubble_server_result *out, uint64_t capacity) {
        uint64_t n = 0;
        while (n < capacity && !results_.empty()) {
            out[n++] = results_.front();
            results_.pop_front();
        }
        return n;
    }

    void stats(bubble_server_stats *s) const {
        std::memset(s, 0, sizeof(*s));
        s->submitted = submitted_;
        s->admitted = admitted_;
        s->completed = completed_;
        s->queued = queue_.size();
        s->active = active_.size();
        s->rounds = rounds_;
        if (!latencies_.empty()) {
            std::vector<double> l = latencies_;
            std::sort(l.begin(), l.end());
            auto pct = [&](double p) {
                const double pos = p * (double)(l.size() - 1);
                const size_t i = (size_t)std::floor(pos);
                const size_t j = std::min(i + 1, l.size() - 1);
                return l[i] + (pos - (double)i) * (l[j] - l[i]);
            };
            s->p50_latency_s = pct(0.50);
            s->p99_latency_s = pct(0.99);
            double sum = 0.0;
            for (double x : l) sum += x;
            s->mean_latency_s = sum / (double)l.size();
            if (last_done_ > first_submit_) s->solves_per_s = (double)completed_ / (last_done_ - first_submit_);
        }
        s->cell_updates = cell_updates_;
    }

   private:
    struct Req {
        uint64_t id = 0;
        bubble_spec spec{};
        uint64_t steps = 0;
        double submit = 0.0;
    };
    struct Active {
        Req req;
        double admit = 0.0;
        uint64_t remaining = 0;
    };
    Server() = default;

    void finish_error(const Req &r, int status) {
        bubble_server_result res;
        std::memset(&res, 0, sizeof(res));
        res.id = r.id;
        res.status = status;
        std::memcpy(res.grid, r.spec.grid, sizeof(res.grid));
        res.steps = r.steps;
        res.submit_s = r.submit;
        res.admit_s = -1.0;
        res.done_s = now();
        results_.push_back(res);
    }

    bubble_server_options opt_{};
    std::unique_ptr<Batch> batch_;
    std::deque<Req> queue_;
    std::unordered_map<uint32_t, Active> active_;
    std::deque<bubble_server_result> results_;
    std::vector<double> latencies_;
    std::chrono::steady_clock::time_point t0_;
    uint64_t next_id_ = 1, submitted_ = 0, admitted_ = 0, completed_ = 0, rounds_ = 0;
    double first_submit_ = -1.0, last_done_ = 0.0, cell_updates_ = 0.0;
};

}  // namespace bubble

struct bubble_server {
    std::unique_ptr<bubble::Server> impl;
};

namespace {
int fail(int code, const std::string &msg) {
    bubble::set_last_error(msg);
    return code;
}
}  // namespace

extern "C" {

void bubble_server_options_default(bubble_server_options *out) {
    if (!out) return;
    out->math = BUBBLE_MATH_FAST;
    out->tile_y = 16;
    out->chunk_steps = 50;
    out->max_active = 64;
    out->memory_fraction = 0.85f;
    out->use_graph = 1;
    out->resident_cells = 0;
    out->policy = BUBBLE_SERVE_FIFO;
    out->chunk_planes = 0;
}

int bubble_server_create(const bubble_server_options *opt, bubble_server **out) {
    if (!out) return fail(BUBBLE_ERR_INVALID, "out is NULL");
    *out = nullptr;
    bubble_server_options o;
    bubble_server_options_default(&o);
    if (opt) o = *opt;
    std::string err;
    std::unique_ptr<bubble::Server> impl;
    const int rc = bubble::Server::create(o, impl, err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    *out = new bubble_server{std::move(impl)};
    return BUBBLE_OK;
}

void bubble_server_destroy(bubble_server *server) { delete server; }

int bubble_server_submit(bubble_server *server, const bubble_spec *spec, uint64_t steps, uint64_t *id) {
    if (!server || !server->impl || !spec || !id) return fail(BUBBLE_ERR_INVALID, "NULL argument");
    std::string err;
    const int rc = server->impl->submit(*spec, steps, id, err);
    return rc == BUBBLE_OK ? rc : fail(rc, err);
}

int bubble_server_tick(bubble_server *server, int32_t *busy) {
    if (!server || !server->impl || !busy) return fail(BUBBLE_ERR_INVALID, "NULL argument");
    std::string err;
    const int rc = server->impl->tick(busy, err);
    return rc == BUBBLE_OK ? rc : fail(rc, err);
}

int bubble_server_run_until_idle(bubble_server *server) {
    if (!server || !server->impl) return fail(BUBBLE_ERR_INVALID, "server is NULL");
    std::string err;
    const int rc = server->impl->run_until_idle(err);
    return rc == BUBBLE_OK ? rc : fail(rc, err);
}

int bubble_server_poll(bubble_server *server, bubble_server_result *out, uint64_t capacity, uint64_t *n_out) {
    if (!server || !server->impl || !n_out) return fail(BUBBLE_ERR_INVALID, "NULL argument");
    *n_out = out ? server->impl->poll(out, capacity) : 0;
    return BUBBLE_OK;
}

int bubble_server_stats_get(const bubble_server *server, bubble_server_stats *out) {
    if (!server || !server->impl || !out) return fail(BUBBLE_ERR_INVALID, "NULL argument");
    server->impl->stats(out);
    return BUBBLE_OK;
}

double bubble_server_now(const bubble_server *server) {
    return server && server->impl ? server->impl->now() : 0.0;
}

}  // extern "C"
