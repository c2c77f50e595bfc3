// extern "C" boundary of the batched form: include/bubble_batch.h.
#include <cstring>
#include <memory>
#include <string>

#include "../../include/bubble_batch.h"
#include "batch.h"
#include "physics.h"

struct bubble_batch {
    std::unique_ptr<bubble::Batch> impl;
};

namespace {
int fail(int code, const std::string &msg) {
    bubble::set_last_error(msg);
    return code;
}
}  // namespace

extern "C" {

void bubble_batch_options_default(bubble_batch_options *out) {
    if (!out) return;
    out->tile_y = 16;
    out->autotune = 1;
    out->use_graph = 1;
    out->max_grid = 0;
}

int bubble_batch_create(const bubble_spec *specs, uint32_t n, const bubble_batch_options *opt,
                        bubble_batch **out) {
    if (!specs || !out) return fail(BUBBLE_ERR_INVALID, "specs and out must be non-NULL");
    *out = nullptr;
    std::string err;
    std::unique_ptr<bubble::Batch> impl;
    const int rc = bubble::Batch::create(specs, n, opt, impl, err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    *out = new bubble_batch{std::move(impl)};
    return BUBBLE_OK;
}

void bubble_batch_destroy(bubble_batch *batch) { delete batch; }

#define BATCH_CALL(expr)                                                                  \
    do {                                                                                  \
        if (!batch || !batch->impl) return fail(BUBBLE_ERR_INVALID, "batch is NULL");     \
        std::string err;                                                                  \
        const int rc = (expr);                                                            \
        if (rc != BUBBLE_OK) return fail(rc, err);                                        \
        return BUBBLE_OK;                                                                 \
    } while (0)

int bubble_batch_advance(bubble_batch *batch, uint64_t n_steps) { BATCH_CALL(batch->impl->advance(n_steps, err)); }
int bubble_batch_diagnostics(bubble_batch *batch, uint32_t index, bubble_diag *out) {
    if (!out) return fail(BUBBLE_ERR_INVALID, "out is NULL");
    BATCH_CALL(batch->impl->diagnostics(index, out, err));
}
int bubble_batch_copy_state(bubble_batch *batch, uint32_t index, float *field, float *fluid) {
    BATCH_CALL(batch->impl->copy_state(index, field, fluid, err));
}
int bubble_batch_load_state(bubble_batch *batch, uint32_t index, const float *field, const float *fluid) {
    BATCH_CALL(batch->impl->load_state(index, field, fluid, err));
}
int bubble_batch_info_get(const bubble_batch *batch, bubble_batch_info *out) {
    if (!batch || !batch->impl || !out) return fail(BUBBLE_ERR_INVALID, "batch and out must be non-NULL");
    batch->impl->info(out);
    return BUBBLE_OK;
}
float bubble_batch_time(const bubble_batch *batch, uint32_t index) {
    if (!batch || !batch->impl || index >= batch->impl->size()) return 0.0f;
    return batch->impl->time(index);
}

int bubble_ext_test_expire_batch_barrier(bubble_batch *batch, int32_t wait_shift) {
    if (!batch || !batch->impl) return fail(BUBBLE_ERR_INVALID, "batch is NULL");
    if (wait_shift < 10 || wait_shift > 32) return fail(BUBBLE_ERR_INVALID, "wait_shift must be 10..32");
    batch->impl->arm_barrier_expiry(wait_shift);
    return BUBBLE_OK;
}

int bubble_autotune_chunk(const uint32_t grid[3], int32_t tile_y, int32_t math, int32_t *lz_out) {
    if (!grid || !lz_out) return fail(BUBBLE_ERR_INVALID, "grid and lz_out must be non-NULL");
    std::string err;
    const int lz = bubble::autotune_chunk(grid, tile_y, math == BUBBLE_MATH_FAST, err);
    if (lz <= 0) return fail(BUBBLE_ERR_CUDA, err.empty() ? "autotune failed" : err);
    *lz_out = lz;
    return BUBBLE_OK;
}

}  // extern "C"
