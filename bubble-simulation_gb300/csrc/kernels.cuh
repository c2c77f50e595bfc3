// CUDA kernels of the lattice time step.
//
//   init_kernel          shaders/init.wgsl:18-26
//   nucleate_kernel      shaders/nucleate.wgsl:59-85
//   prim_kernel          shaders/primitives.wgsl:16-23   (reference-structured path)
//   stage_ref_kernel     shaders/step.wgsl:92-174         (reference-structured path)
//   diag_kernel          shaders/reduce.wgsl:49-140, single pass, FP64 sums
//
// This header is included by translation units that differ only in their
// arithmetic flags (see physics.cuh); every template here is instantiated
// there.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "params.h"
#include "physics.cuh"

namespace bubble {
namespace dev {

// wrap1 (shaders/common.wgsl:80-89): reach <= 2 with n >= 8, one add suffices.
BUBBLE_DEV int wrap1(int i, int n) {
    int r = i;
    if (r < 0) r += n;
    if (r >= n) r -= n;
    return r;
}

template <typename R>
BUBBLE_DEV size_t cell_index(int x, int y, int z, const LatticeParams<R> &P) {
    return ((size_t)z * (size_t)P.ny + (size_t)y) * (size_t)P.nx + (size_t)x;
}

// ---------------------------------------------------------------------------
//  init (shaders/init.wgsl:18-26): phi = pi = 0, E = e_ref, Z = 0
// ---------------------------------------------------------------------------
template <typename R>
__global__ void init_kernel(V2<R> *__restrict__ field, V4<R> *__restrict__ fluid, uint64_t n,
                            R e_ref) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        field[i] = V2<R>{R(0), R(0)};
        fluid[i] = V4<R>{e_ref, R(0), R(0), R(0)};
    }
}

// ---------------------------------------------------------------------------
//  nucleate (shaders/nucleate.wgsl:59-85)
// ---------------------------------------------------------------------------
// phi <- max(phi, phi_b/2 (1 - tanh((r - r0 dx) / l_w))) over the batch, r the
// minimum-image distance from the integer cell position.  As in the
// reference the max reaches every cell: a bubble farther than the tanh
// cut-off contributes exactly 0 (det_tanh_r rounds to 1 there), so those
// terms are max(phi, 0) without evaluating tanh.
// Bubbles travel as a by-value kernel parameter (constant bank, broadcast
// to the warp), so a nucleation launch needs no staging copy; larger batches
// are split over several launches, which gives the same result because max()
// is exact and order-independent.
constexpr int kNucleateBatch = 128;
struct BubbleBatch {
    int32_t count;
    int32_t _pad[3];
    V4<float> b[kNucleateBatch];
};

// The launch covers the lattice in bricks of 32 x 8 x 8 cells, one CTA
// each.  The CTA first keeps the bubbles that can reach its brick: a lower
// bound of every cell's distance (per axis the circular distance of the
// brick's centre minus its half extent -- the periodic distance is
// 1-Lipschitz) whose tanh argument exceeds the cut-off by a margin rules a
// bubble out, its profile being exactly 0 in the whole brick.  Every cell
// then takes max(phi, 0), the far field of all the batch's bubbles, and the
// maximum over the kept bubbles alone, in any order: the result equals the
// reference's loop over the whole batch bit for bit.  A cell whose value
// does not change is not written back.
constexpr int kNucBx = 32, kNucBy = 8, kNucBz = 8;

template <typename R>
__global__ void __launch_bounds__(256) nucleate_kernel(V2<R> *__restrict__ field,
                                                        const __grid_constant__ BubbleBatch batch,
                                                        LatticeParams<R> P) {
    __shared__ int kept[kNucleateBatch];
    __shared__ int n_kept;
    const int bx = blockIdx.x * kNucBx, by = blockIdx.y * kNucBy, bz = blockIdx.z * kNucBz;
    const int ex = min(kNucBx, P.nx - bx), ey = min(kNucBy, P.ny - by), ez = min(kNucBz, P.nz - bz);
    if (threadIdx.x == 0) n_kept = 0;
    __syncthreads();
    const R cut = TanhCut<R>::value;
    for (int b = threadIdx.x; b < batch.count; b += blockDim.x) {
        const V4<float> bub = batch.b[b];
        const double c[3] = {(double)bub.x, (double)bub.y, (double)bub.z};
        const int b0[3] = {bx, by, bz}, e[3] = {ex, ey, ez}, n[3] = {P.nx, P.ny, P.nz};
        double lb2 = 0.0;
        for (int a = 0; a < 3; ++a) {
            const double half = 0.5 * (double)(e[a] - 1);
            double d = (double)b0[a] + half - c[a];
            if (d > 0.5 * n[a]) d -= n[a];
            if (d < -0.5 * n[a]) d += n[a];
            const double g = fmax(fabs(d) - half, 0.0);
            lb2 += g * g;
        }
        const double arg_lb = (sqrt(lb2) * (double)P.dx - (double)bub.w * (double)P.dx) / (double)P.wall_width;
        if (!(arg_lb > (double)cut + 0.25)) kept[atomicAdd(&n_kept, 1)] = b;
    }
    __syncthreads();
    const int nk = n_kept;
    const int tx = threadIdx.x % kNucBx, ty = threadIdx.x / kNucBx;
    if (tx >= ex || ty >= ey) return;
    const R nxr = R(P.nx), nyr = R(P.ny), nzr = R(P.nz);
    const R px = R(bx + tx), py = R(by + ty);
    for (int zz = 0; zz < ez; ++zz) {
        const int z = bz + zz;
        const size_t i = cell_index(bx + tx, by + ty, z, P);
        const R phi0 = field[i].x;
        R phi = vmax(phi0, R(0));
        const R pz = R(z);
        for (int q = 0; q < nk; ++q) {
            const V4<float> bub = batch.b[kept[q]];
            const R dx = min_image(px - R(bub.x), nxr);
            const R dy = min_image(py - R(bub.y), nyr);
            const R dz = min_image(pz - R(bub.z), nzr);
            const R r = sqrt(dx * dx + dy * dy + dz * dz) * P.dx;
            const R arg = (r - R(bub.w) * P.dx) / P.wall_width;
            R profile = R(0);
            if (!(arg > cut)) profile = R(0.5) * P.phi_b * (R(1.0) - det_tanh_r<R>(arg));
            phi = vmax(phi, profile);
        }
        bool same;
        if constexpr (sizeof(R) == 4) same = __float_as_uint((float)phi) == __float_as_uint((float)phi0);
        else same = __double_as_longlong((double)phi) == __double_as_longlong((double)phi0);
        if (!same) field[i].x = phi;
    }
}

// ---------------------------------------------------------------------------
//  Reference-structured path: primitives pass + stage pass
// ---------------------------------------------------------------------------
template <typename R>
__global__ void prim_kernel(const V4<R> *__restrict__ fluid, V4<R> *__restrict__ prim, uint64_t n,
                            LatticeParams<R> P) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        prim[i] = prim_from_cons<R, false>(fluid[i], P);
}

// One thread per cell, two HLL fluxes per axis, every operand read from
// global memory: the reference's own kernel structure (step.wgsl:92-174).
template <typename R>
__global__ void stage_ref_kernel(StageArgs<R> A, const V4<R> *__restrict__ prim,
                                 LatticeParams<R> P) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int z = blockIdx.z;
    if (x >= P.nx) return;
    const R zmax2 = P.z_max * P.z_max;
    const size_t i0 = cell_index(x, y, z, P);
    const V2<R> f0 = A.field_in[i0];
    const R phi0 = f0.x, pi0 = f0.y;
    const V4<R> q0 = sanitise(prim[i0], P.p_floor, zmax2);
    R lap_sum = R(0);
    R grad[3] = {R(0), R(0), R(0)};
    V4<R> fd{R(0), R(0), R(0), R(0)};
#pragma unroll
    for (int axis = 0; axis < 3; ++axis) {
        const int ex = axis == 0, ey = axis == 1, ez = axis == 2;
        const size_t im1 = cell_index(wrap1(x - ex, P.nx), wrap1(y - ey, P.ny), wrap1(z - ez, P.nz), P);
        const size_t ip1 = cell_index(wrap1(x + ex, P.nx), wrap1(y + ey, P.ny), wrap1(z + ez, P.nz), P);
        const size_t im2 =
            cell_index(wrap1(x - 2 * ex, P.nx), wrap1(y - 2 * ey, P.ny), wrap1(z - 2 * ez, P.nz), P);
        const size_t ip2 =
            cell_index(wrap1(x + 2 * ex, P.nx), wrap1(y + 2 * ey, P.ny), wrap1(z + 2 * ez, P.nz), P);
        const R phi_m = A.field_in[im1].x;
        const R phi_p = A.field_in[ip1].x;
        lap_sum = lap_sum + (phi_m + phi_p - R(2.0) * phi0);
        grad[axis] = R(0.5) * (phi_p - phi_m) * P.inv_dx;
        const V4<R> qm2 = sanitise(prim[im2], P.p_floor, zmax2);
        const V4<R> qm1 = sanitise(prim[im1], P.p_floor, zmax2);
        const V4<R> qp1 = sanitise(prim[ip1], P.p_floor, zmax2);
        const V4<R> qp2 = sanitise(prim[ip2], P.p_floor, zmax2);
        const V4<R> s_m1 = limit_slope4(v4_sub(qm1, qm2), v4_sub(q0, qm1));
        const V4<R> s_0 = limit_slope4(v4_sub(q0, qm1), v4_sub(qp1, q0));
        const V4<R> s_p1 = limit_slope4(v4_sub(qp1, q0), v4_sub(qp2, qp1));
        const V4<R> lm = sanitise(half_step(qm1, s_m1, R(1)), P.p_floor, zmax2);
        const V4<R> rm = sanitise(half_step(q0, s_0, R(-1)), P.p_floor, zmax2);
        const V4<R> lp = sanitise(half_step(q0, s_0, R(1)), P.p_floor, zmax2);
        const V4<R> rp = sanitise(half_step(qp1, s_p1, R(-1)), P.p_floor, zmax2);
        V4<R> fm, fp;
        if (axis == 0) {
            fm = hll_flux<0, R, false>(lm, rm, zmax2, P);
            fp = hll_flux<0, R, false>(lp, rp, zmax2, P);
        } else if (axis == 1) {
            fm = hll_flux<1, R, false>(lm, rm, zmax2, P);
            fp = hll_flux<1, R, false>(lp, rp, zmax2, P);
        } else {
            fm = hll_flux<2, R, false>(lm, rm, zmax2, P);
            fp = hll_flux<2, R, false>(lp, rp, zmax2, P);
        }
        fd.x = fd.x + (fp.x - fm.x) * P.inv_dx;
        fd.y = fd.y + (fp.y - fm.y) * P.inv_dx;
        fd.z = fd.z + (fp.z - fm.z) * P.inv_dx;
        fd.w = fd.w + (fp.w - fm.w) * P.inv_dx;
    }
    const R laplacian = lap_sum * P.inv_dx * P.inv_dx;
    const R vv = q0.x * q0.x + q0.y * q0.y + q0.z * q0.z;
    const R gam = R(1.0) / sqrt(vmax(R(1.0) - vv, R(1e-12)));
    const R dphi_proper = gam * (pi0 + (q0.x * grad[0] + q0.y * grad[1] + q0.z * grad[2]));
    const R drag = P.eta * dphi_proper;
    const R d_phi = pi0;
    const R d_pi = laplacian - dpotential(phi0, P) - drag;
    const R dE = -fd.x + drag * pi0;
    const R dZx = -fd.y - drag * grad[0];
    const R dZy = -fd.z - drag * grad[1];
    const R dZz = -fd.w - drag * grad[2];
    const V4<R> u_in = A.fluid_in[i0];
    const V2<R> fu{f0.x + A.dt * d_phi, f0.y + A.dt * d_pi};
    const V4<R> uu{u_in.x + A.dt * dE, u_in.y + A.dt * dZx, u_in.z + A.dt * dZy,
                   u_in.w + A.dt * dZz};
    if (A.stage == 0) {
        A.field_out[i0] = V2<R>{A.a1 * fu.x, A.a1 * fu.y};
        A.fluid_out[i0] = V4<R>{A.a1 * uu.x, A.a1 * uu.y, A.a1 * uu.z, A.a1 * uu.w};
    } else {
        const V2<R> fn = A.field_n[i0];
        const V4<R> un = A.fluid_n[i0];
        A.field_out[i0] = V2<R>{A.a0 * fn.x + A.a1 * fu.x, A.a0 * fn.y + A.a1 * fu.y};
        A.fluid_out[i0] = V4<R>{A.a0 * un.x + A.a1 * uu.x, A.a0 * un.y + A.a1 * uu.y,
                                A.a0 * un.z + A.a1 * uu.z, A.a0 * un.w + A.a1 * uu.w};
    }
}

// ---------------------------------------------------------------------------
//  Diagnostics (shaders/reduce.wgsl:49-140), one pass, FP64 sums
// ---------------------------------------------------------------------------
// Per-cell terms in the state precision exactly as cell_contribution; sums in
// FP64.  Every block writes its partial to `partials`; the last block to
// finish (ticket counter) folds them in a fixed order, writes `out` and
// re-arms the counter, so the result does not depend on block timing.
constexpr int kDiagThreads = 256;
constexpr int kDiagMaxBlocks = 1024;

struct DiagPartial {
    double s[4];
    float vmax;
    uint32_t nonfinite;
    uint32_t _pad[2];
};

template <typename R>
BUBBLE_DEV double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename R, int MIXED>
__global__ void __launch_bounds__(kDiagThreads)
    diag_kernel(const V2<R> *__restrict__ field, const V4<R> *__restrict__ fluid,
                LatticeParams<R> P, DiagPartial *__restrict__ partials,
                unsigned int *__restrict__ ticket, DiagResult *__restrict__ out) {
    const uint64_t n = (uint64_t)P.nx * P.ny * P.nz;
    const uint64_t xy = (uint64_t)P.nx * P.ny;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    float vmaxv = 0.0f;
    uint32_t bad = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int z = (int)(i / xy);
        const int rem = (int)(i - (uint64_t)z * xy);
        const int y = rem / P.nx;
        const int x = rem - y * P.nx;
        const V2<R> f = field[i];
        const R phi = f.x, pi = f.y;
        R grad2 = R(0);
        {
            const R d = R(0.5) *
                        (field[cell_index(wrap1(x + 1, P.nx), y, z, P)].x -
                         field[cell_index(wrap1(x - 1, P.nx), y, z, P)].x) *
                        P.inv_dx;
            grad2 = grad2 + d * d;
        }
        {
            const R d = R(0.5) *
                        (field[cell_index(x, wrap1(y + 1, P.ny), z, P)].x -
                         field[cell_index(x, wrap1(y - 1, P.ny), z, P)].x) *
                        P.inv_dx;
            grad2 = grad2 + d * d;
        }
        {
            const R d = R(0.5) *
                        (field[cell_index(x, y, wrap1(z + 1, P.nz), P)].x -
                         field[cell_index(x, y, wrap1(z - 1, P.nz), P)].x) *
                        P.inv_dx;
            grad2 = grad2 + d * d;
        }
        const V4<R> u = fluid[i];
        // In the perturbation form e_lab is max(E, e_floor) - e_bg: the sums of
        // e_total and e_lab then miss N e_bg, which the host adds in FP64.
        const R e_lab = vmax(u.x, P.e_floor);
        const V4<R> q = recover<R, false, MIXED>(u, P, phi);
        const R v2 = q.x * q.x + q.y * q.y + q.z * q.z;
        // the thermal form's field holds V(phi, 0); the rest of V(phi, T) is in E
        R pot;
        if constexpr (MIXED == kThermal) pot = thermal_potential0(phi, P);
        else pot = potential(phi, P);
        const R e_total = R(0.5) * pi * pi + R(0.5) * grad2 + pot + e_lab;
        const R broken = phi > R(0.5) * P.phi_b ? R(1.0) : R(0.0);
        R kinetic;
        if constexpr (MIXED == kPert) kinetic = ((e_lab + q.w) + (P.e_bg + P.p_bg)) * v2;
        else kinetic = (e_lab + q.w) * v2;
        acc[0] += (double)e_total;
        acc[1] += (double)broken;
        acc[2] += (double)kinetic;
        acc[3] += (double)e_lab;
        const float vl = (float)sqrt(v2);
        // max(E, e_floor) hides a NaN in E, so the raw state is checked too.
        if (!isfinite(e_total) || !isfinite(vl) || !isfinite(f.x + f.y + u.x + u.y + u.z + u.w)) bad = 1;
        vmaxv = fmaxf(vmaxv, vl);
    }
    __shared__ double sh[kDiagThreads / 32][4];
    __shared__ float shm[kDiagThreads / 32];
    __shared__ uint32_t shb[kDiagThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = warp_sum<R>(acc[k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vmaxv = fmaxf(vmaxv, __shfl_xor_sync(0xffffffffu, vmaxv, o));
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) {
        for (int k = 0; k < 4; ++k) sh[w][k] = acc[k];
        shm[w] = vmaxv;
        shb[w] = bad;
    }
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) {
        DiagPartial pt;
        for (int k = 0; k < 4; ++k) {
            double s = 0.0;
            for (int q = 0; q < kDiagThreads / 32; ++q) s += sh[q][k];
            pt.s[k] = s;
        }
        float m = 0.0f;
        uint32_t b = 0;
        for (int q = 0; q < kDiagThreads / 32; ++q) {
            m = fmaxf(m, shm[q]);
            b |= shb[q];
        }
        pt.vmax = m;
        pt.nonfinite = b;
        pt._pad[0] = pt._pad[1] = 0;
        partials[blockIdx.x] = pt;
        __threadfence();
        const unsigned int prev = atomicAdd(ticket, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // Fold the partials: thread k sums partials k, k+256, ... in order, then
    // a fixed tree over the 256 threads.
    __shared__ double fold[kDiagThreads][4];
    __shared__ float foldm[kDiagThreads];
    __shared__ uint32_t foldb[kDiagThreads];
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    float m = 0.0f;
    uint32_t b = 0;
    for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) {
        const volatile DiagPartial *pp = partials + q;
        for (int k = 0; k < 4; ++k) s[k] += pp->s[k];
        m = fmaxf(m, pp->vmax);
        b |= pp->nonfinite;
    }
    for (int k = 0; k < 4; ++k) fold[threadIdx.x][k] = s[k];
    foldm[threadIdx.x] = m;
    foldb[threadIdx.x] = b;
    __syncthreads();
    for (int h = kDiagThreads / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            for (int k = 0; k < 4; ++k) fold[threadIdx.x][k] += fold[threadIdx.x + h][k];
            foldm[threadIdx.x] = fmaxf(foldm[threadIdx.x], foldm[threadIdx.x + h]);
            foldb[threadIdx.x] |= foldb[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < 4; ++k) out->sums[k] = fold[0][k];
        out->max_v_bits = __float_as_uint(foldm[0]);
        out->nonfinite = foldb[0];
        out->cells = n;
        *ticket = 0u;  // re-arm for the next launch on this scratch
    }
}

inline int diag_blocks(uint64_t n) {
    uint64_t b = (n + kDiagThreads - 1) / kDiagThreads;
    if (b > (uint64_t)kDiagMaxBlocks) b = kDiagMaxBlocks;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace dev
}  // namespace bubble
