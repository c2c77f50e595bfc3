// Staging helpers of the fused stage kernels: compile-time loops, mbarrier
// and TMA (cp.async.bulk.tensor) primitives, per-element cp.async copies.
//
// Every mbarrier wait here is bounded by a clock limit, so a copy that never
// completes turns into an error status instead of a hung CTA.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "kernels.cuh"
#include "tma.h"

namespace bubble {
namespace dev {

// Compile-time loop: f(std::integral_constant<int, I>{}) for I = I0 .. N-1.
template <int I0, int N, typename F>
BUBBLE_DEV void static_for(F &&f) {
    if constexpr (I0 < N) {
        f(std::integral_constant<int, I0>{});
        static_for<I0 + 1, N>(f);
    }
}

BUBBLE_DEV uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

BUBBLE_DEV void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
BUBBLE_DEV void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
BUBBLE_DEV void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
BUBBLE_DEV void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
BUBBLE_DEV bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after 2^shift SM cycles (2^31 by default, about a
// second at GB300 clocks).
BUBBLE_DEV bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int shift) {
    const long long start = clock64();
    const long long limit = 1ll << shift;
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - start > limit) return false;
    }
    return true;
}
BUBBLE_DEV void tma_load_4d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
}
BUBBLE_DEV void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
        : "memory");
}
BUBBLE_DEV void cp_async_16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
BUBBLE_DEV void cp_async_8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
BUBBLE_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
BUBBLE_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// all but the most recent committed group complete
BUBBLE_DEV void cp_async_wait_but_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

template <typename R>
BUBBLE_DEV void cp_async_v4(V4<R> *dst, const V4<R> *src) {
    if constexpr (sizeof(R) == 4) {
        cp_async_16(dst, src);
    } else {
        cp_async_16(dst, src);
        cp_async_16(reinterpret_cast<char *>(dst) + 16, reinterpret_cast<const char *>(src) + 16);
    }
}
template <typename R>
BUBBLE_DEV void cp_async_v2(V2<R> *dst, const V2<R> *src) {
    if constexpr (sizeof(R) == 4) cp_async_8(dst, src);
    else cp_async_16(dst, src);
}

constexpr int pad32(int n) { return (n + 31) / 32 * 32; }
constexpr int round_up(int n, int m) { return (n + m - 1) / m * m; }
constexpr size_t align128(size_t b) { return (b + 127) / 128 * 128; }

}  // namespace dev
}  // namespace bubble
