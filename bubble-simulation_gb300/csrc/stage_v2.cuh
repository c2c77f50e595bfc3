// Fused SSP-RK3 stage kernel with asynchronous plane staging.
//
// Same arithmetic as stage_fused_kernel (shaders/primitives.wgsl +
// shaders/step.wgsl:92-174, each face flux computed once), reorganised so
// that no thread waits on a global load inside the z-march:
//
//   * Raw planes of U_in are staged into shared memory one iteration ahead.
//     Tiles whose halo lies inside the lattice use the Tensor Memory
//     Accelerator (cp.async.bulk.tensor, completion on an mbarrier); tiles
//     on the periodic boundary, and lattices whose row pitch TMA cannot
//     address, use per-element cp.async with wrapped addresses.
//   * The own-cell U_in and U^n needed by the stage combine are loaded into
//     registers one phase before they are used.
//   * Two barriers per plane.  Phase X(z) combines plane z-1 and computes
//     the limited face states of plane z; phase Y(z) recovers primitives of
//     plane z+3 from the staged raw plane and computes the face fluxes of
//     plane z.
//
// Every mbarrier wait is bounded by a clock limit; on expiry the CTA sets
// bit 0 of *status, waits (bounded) for its own copy in flight and returns.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "kernels.cuh"
#include "staging.cuh"
#include "tma.h"

namespace bubble {
namespace dev {

template <typename R, int TY>
struct V2Layout {
    static constexpr int TX = 32;
    static constexpr int PW = TX + 4, PH = TY + 4, PC = PW * PH, NC = TX * TY;
    // TY = 16 (640 threads, one CTA per SM) was measured no faster than TY = 8
    // at 512^3 (17.09 vs 17.01 ms per step): the smaller halo share is lost to
    // barrier waits with no second CTA to issue from.
    static constexpr int NT = TY == 16 ? 640 : (TY == 8 ? 320 : 192);
    static constexpr int MIN_BLOCKS = (sizeof(R) == 4 && TY <= 8) ? 2 : 1;
    // phase X: combine of the previous plane, then face states
    static constexpr int X_C = NC, X_Z = NC, X_Y = TX * (TY + 2), X_X = (TX + 2) * TY;
    static constexpr int X_TOTAL = X_C + X_Z + X_Y + X_X;
    // Where it costs no extra slot, each kind of phase-X item starts at a
    // multiple of NT, so every unrolled slot holds one kind and the phase's
    // code holds each item body once.
    static constexpr bool X_ALIGN = round_up(X_C, NT) + round_up(X_Z, NT) + round_up(X_Y, NT) + X_X <=
                                    round_up(X_TOTAL, NT);
    static constexpr int XO_Z = X_ALIGN ? round_up(X_C, NT) : X_C;
    static constexpr int XO_Y = XO_Z + (X_ALIGN ? round_up(X_Z, NT) : X_Z);
    static constexpr int XO_X = XO_Y + (X_ALIGN ? round_up(X_Y, NT) : X_Y);
    static constexpr int X_END = XO_X + X_X;
    // phase Y: primitives of the staged plane, then face fluxes
    static constexpr int A_REAL = TY * PW + 4 * TX;
    static constexpr int Y_A = pad32(A_REAL), Y_Z = NC, Y_Y = TX * (TY + 1), Y_X = (TX + 1) * TY;
    static constexpr int Y_TOTAL = Y_A + Y_Z + Y_Y + Y_X;
    static constexpr int PRIM_RING = 4, PHI_RING = 5;
    // shared memory map (bytes)
    static constexpr size_t o_rawu = 0;
    static constexpr size_t o_rawf = align128(o_rawu + 2 * PC * sizeof(V4<R>));
    static constexpr size_t o_prim = align128(o_rawf + 2 * PC * sizeof(V2<R>));
    static constexpr size_t o_phi = align128(o_prim + PRIM_RING * PC * sizeof(V4<R>));
    static constexpr size_t o_xlo = align128(o_phi + PHI_RING * PC * sizeof(R));
    static constexpr size_t o_xhi = o_xlo + TY * (TX + 2) * sizeof(V4<R>);
    static constexpr size_t o_ylo = o_xhi + TY * (TX + 2) * sizeof(V4<R>);
    static constexpr size_t o_yhi = o_ylo + (TY + 2) * TX * sizeof(V4<R>);
    static constexpr size_t o_zlo = o_yhi + (TY + 2) * TX * sizeof(V4<R>);
    static constexpr size_t o_zhi = o_zlo + NC * sizeof(V4<R>);
    static constexpr size_t o_fx = o_zhi + 2 * NC * sizeof(V4<R>);
    static constexpr size_t o_fy = o_fx + TY * (TX + 1) * sizeof(V4<R>);
    static constexpr size_t o_fz = o_fy + (TY + 1) * TX * sizeof(V4<R>);
    static constexpr size_t o_bar = o_fz + 2 * NC * sizeof(V4<R>);
    static constexpr size_t bytes = o_bar + 2 * sizeof(uint64_t);
    static constexpr uint32_t plane_tx_bytes = PC * (sizeof(V4<R>) + sizeof(V2<R>));
    static_assert(NT >= NC, "the combine phase maps one thread per column");
    static_assert(X_C % 32 == 0 && XO_Z % 32 == 0 && (XO_Z + X_Z) % 32 == 0 && XO_Y % 32 == 0 &&
                      (XO_Y + X_Y) % 32 == 0 && XO_X % 32 == 0,
                  "warp-uniform X");
    static_assert(Y_A % 32 == 0 && (Y_A + Y_Z) % 32 == 0 && (Y_A + Y_Z + Y_Y) % 32 == 0, "warp-uniform Y");
};

// Cross-shaped halo item k of a plane -> smem (i, j).
template <int TX, int TY, int PW>
BUBBLE_DEV void cross_item(int k, int &i, int &j) {
    constexpr int band = TY * PW;
    if (k < band) {
        j = 2 + k / PW;
        i = k - (j - 2) * PW;
    } else {
        const int kk = k - band;
        const int r = kk / TX;
        j = r < 2 ? r : TY + r;
        i = 2 + (kk - r * TX);
    }
}

// One work item: the column tile `tile_xy` of lattice P, z chunk `chunk`
// (planes [chunk*lz, min((chunk+1)*lz, nz))), one RK stage.  Returns false
// when a bounded wait expired (bit 0 of *status is set); the CTA must then
// stop.  Usable repeatedly by one CTA: it starts with a barrier and leaves
// no copy in flight.
// QBP: planes whose prologue loads are issued together (FP32; FP64 stages
// one at a time).
template <typename R, bool FAST, int MIXED, int TY, int QBP = 4>
BUBBLE_DEV bool v2_item(unsigned char *smem, const StageArgs<R> &A, const LatticeParams<R> &P, int lz,
                        const StageMaps *maps, int tma_ok, int *status, int tile_xy, int chunk) {
    using L = V2Layout<R, TY>;
    constexpr int TX = L::TX, NT = L::NT, PW = L::PW, PC = L::PC, NC = L::NC;
    __syncthreads();  // a previous item on this CTA is done with shared memory
    V4<R> *raw_u = reinterpret_cast<V4<R> *>(smem + L::o_rawu);
    V2<R> *raw_f = reinterpret_cast<V2<R> *>(smem + L::o_rawf);
    V4<R> *prim_s = reinterpret_cast<V4<R> *>(smem + L::o_prim);
    R *phi_s = reinterpret_cast<R *>(smem + L::o_phi);
    V4<R> *xlo = reinterpret_cast<V4<R> *>(smem + L::o_xlo);
    V4<R> *xhi = reinterpret_cast<V4<R> *>(smem + L::o_xhi);
    V4<R> *ylo = reinterpret_cast<V4<R> *>(smem + L::o_ylo);
    V4<R> *yhi = reinterpret_cast<V4<R> *>(smem + L::o_yhi);
    V4<R> *zlo = reinterpret_cast<V4<R> *>(smem + L::o_zlo);
    V4<R> *zhi = reinterpret_cast<V4<R> *>(smem + L::o_zhi);
    V4<R> *fxs = reinterpret_cast<V4<R> *>(smem + L::o_fx);
    V4<R> *fys = reinterpret_cast<V4<R> *>(smem + L::o_fy);
    V4<R> *fzs = reinterpret_cast<V4<R> *>(smem + L::o_fz);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::o_bar);

    const int t = threadIdx.x;
    const int ntx = (P.nx + TX - 1) / TX;
    const int x0 = (tile_xy % ntx) * TX;
    const int y0 = (tile_xy / ntx) * TY;
    const int z0 = chunk * lz;
    const int z1 = min(z0 + lz, P.nz);
    const int xe = min(TX, P.nx - x0);
    const int ye = min(TY, P.ny - y0);
    const R zmax2 = P.z_max * P.z_max;
    const size_t plane = (size_t)P.nx * (size_t)P.ny;
    const bool tma = tma_ok && x0 >= 2 && x0 + TX + 2 <= P.nx && y0 >= 2 && y0 + TY + 2 <= P.ny;
    const int zlast = z1 + 1;  // last plane whose primitives are needed

    auto prim_slot = [&](int p) { return prim_s + ((p + 8) & (L::PRIM_RING - 1)) * PC; };
    auto phi_slot = [&](int p) { return phi_s + ((p + 10) % L::PHI_RING) * PC; };
    auto raw_slot = [&](int p) { return (p - (z0 + 3)) & 1; };

    if (tma && t == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }

    // ---- static work plan --------------------------------------------------
    // Thread t takes the items k = t + r NT (r = 0, 1, ...) of each phase, the
    // same on every plane.  The kinds of item are contiguous ranges of k, so
    // the slot r meets only the kinds whose range intersects [r NT, (r+1) NT):
    // with r unrolled those are known at compile time, and each item's indices
    // are decoded once here instead of on every plane.
    constexpr int NRX = (L::X_END + NT - 1) / NT;
    constexpr int NRY = (L::Y_TOTAL + NT - 1) / NT;
    constexpr int NRA = (L::A_REAL + NT - 1) / NT;  // slots holding staged cells
    // own cell of the combine (k = t < NC)
    const int ci = t % TX, cj = t / TX;
    const bool c_valid = t < NC && ci < xe && cj < ye;
    const int cc = (cj + 2) * PW + (ci + 2);
    const uint32_t c_off = (uint32_t)(y0 + cj) * (uint32_t)P.nx + (uint32_t)(x0 + ci);
    // Staged cells (the Y-phase primitive items and the per-element copies):
    // ya_c = the cell in the cross-shaped halo layout, -1 outside the tile's
    // cells; ya_g = the same cell within a lattice plane, periodic wrap applied.
    int ya_c[NRY];
    uint32_t ya_g[NRA];
    static_for<0, NRY>([&](auto rc) {
        constexpr int r = decltype(rc)::value;
        ya_c[r] = -1;
        if constexpr (r < NRA) {
            ya_g[r] = 0;
            const int k = t + r * NT;
            if (k < L::A_REAL) {
                int i, j;
                cross_item<TX, TY, PW>(k, i, j);
                if (i < xe + 4 && j < ye + 4) {
                    ya_c[r] = j * PW + i;
                    ya_g[r] = (uint32_t)wrap1(y0 - 2 + j, P.ny) * (uint32_t)P.nx + (uint32_t)wrap1(x0 - 2 + i, P.nx);
                }
            }
        }
    });

    // Stage raw plane p (p >= z0+3) asynchronously.
    auto issue = [&](int p) {
        const int s = raw_slot(p);
        const int gz = wrap1(p, P.nz);
        if (tma) {
            if (t == 0) {
                fence_proxy_async();
                if (A.test_tx != 0 && p == z0 + 3) {
                    // test hook: bytes that no copy delivers, and no copy issued
                    mbar_expect_tx(&bar[s], A.test_tx);
                } else {
                    mbar_expect_tx(&bar[s], L::plane_tx_bytes);
                    tma_load_4d(raw_u + s * PC, &maps->fluid, &bar[s], 0, x0 - 2, y0 - 2, gz);
                    tma_load_3d(raw_f + s * PC, &maps->field, &bar[s], 2 * (x0 - 2), y0 - 2, gz);
                }
            }
        } else {
            const size_t base = (size_t)gz * plane;
            static_for<0, NRA>([&](auto rc) {
                constexpr int r = decltype(rc)::value;
                const int c = ya_c[r];
                if (c >= 0) {
                    cp_async_v4(raw_u + s * PC + c, A.fluid_in + base + ya_g[r]);
                    cp_async_v2(raw_f + s * PC + c, A.field_in + base + ya_g[r]);
                }
            });
            cp_async_commit();
        }
    };
    // Wait for raw plane p; returns false when the bounded wait expired.
    auto wait_plane = [&](int p) -> bool {
        if (tma) {
            const uint32_t parity = ((p - (z0 + 3)) >> 1) & 1;
            return mbar_wait_bounded(&bar[raw_slot(p)], parity, A.wait_shift);
        }
        cp_async_wait_all();
        return true;
    };

    // Synchronous staging of the prologue: the loads of NQ <= QB planes
    // p .. p+NQ-1 are all issued before the first is used.
    constexpr int QB = sizeof(R) == 4 ? QBP : 1;
    static_assert(4 % QB == 0, "the prologue stages four planes");
    struct Staged {
        V4<R> u[QB][NRA];
        R phi[QB][NRA];
    };
    auto load_planes = [&](int p, Staged &S, auto nq) {
        constexpr int NQ = decltype(nq)::value;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const size_t base = (size_t)wrap1(p + q, P.nz) * plane;
            static_for<0, NRA>([&](auto rc) {
                constexpr int r = decltype(rc)::value;
                if (ya_c[r] >= 0) {
                    S.u[q][r] = A.fluid_in[base + ya_g[r]];
                    S.phi[q][r] = A.field_in[base + ya_g[r]].x;
                }
            });
        }
    };
    auto store_planes = [&](int p, const Staged &S, auto nq) {
        constexpr int NQ = decltype(nq)::value;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            V4<R> *pr = prim_slot(p + q);
            R *ph = phi_slot(p + q);
            static_for<0, NRA>([&](auto rc) {
                constexpr int r = decltype(rc)::value;
                const int c = ya_c[r];
                if (c >= 0) {
                    ph[c] = S.phi[q][r];
                    pr[c] = recover_sanitised<R, FAST, MIXED>(S.u[q][r], P, S.phi[q][r], zmax2);
                }
            });
        }
    };
    auto z_states = [&](int p, int n, V4<R> &lo, V4<R> &hi) {
        const int i = n % TX, j = n / TX;
        const int c = (j + 2) * PW + (i + 2);
        face_states<R, FAST>(prim_slot(p - 1)[c], prim_slot(p)[c], prim_slot(p + 1)[c], P.p_floor, zmax2, lo, hi);
    };

    // ---- prologue ----------------------------------------------------------
    // Planes z0-2 .. z0+1 fill the 4-slot primitive ring; the z face
    // z0 - 1/2 needs all four.  Plane z0+2 then takes the slot of z0-2: its
    // loads are in flight while that face is computed.
    {
        Staged S;
        for (int p = z0 - 2; p <= z0 + 1; p += QB) {
            load_planes(p, S, std::integral_constant<int, QB>{});
            store_planes(p, S, std::integral_constant<int, QB>{});
        }
    }
    Staged S2;
    load_planes(z0 + 2, S2, std::integral_constant<int, 1>{});
    __syncthreads();  // also publishes the mbarrier initialisation
    for (int n = t; n < NC; n += NT) {
        V4<R> lo_m, hi_m, lo_0, hi_0;
        z_states(z0 - 1, n, lo_m, hi_m);
        z_states(z0, n, lo_0, hi_0);
        zhi[((z0 + 8) & 1) * NC + n] = hi_0;
        R phl = R(0), phr = R(0);
        if constexpr (MIXED == kThermal) {
            const int c = (n / TX + 2) * PW + (n % TX + 2);
            phl = phi_slot(z0 - 1)[c];
            phr = phi_slot(z0)[c];
        }
        fzs[((z0 - 1 + 8) & 1) * NC + n] = hll_flux<2, R, FAST, MIXED>(hi_m, lo_0, zmax2, P, phl, phr);
    }
    __syncthreads();
    store_planes(z0 + 2, S2, std::integral_constant<int, 1>{});
    if (z0 + 3 <= zlast) issue(z0 + 3);
    __syncthreads();

    // own-cell state of the plane awaiting its combine, loaded a phase ahead
    V2<R> pf{R(0), R(0)}, pfn{R(0), R(0)};
    V4<R> pu{R(0), R(0), R(0), R(0)}, pun{R(0), R(0), R(0), R(0)};

    for (int z = z0;; ++z) {
        // ring slots of this plane, computed once for every item
        const V4<R> *pr_zm1 = prim_slot(z - 1), *pr_z = prim_slot(z);
        const V4<R> *pr_zp1 = prim_slot(z + 1), *pr_zp2 = prim_slot(z + 2);
        const R *ph_zm2 = phi_slot(z - 2), *ph_zm1 = phi_slot(z - 1), *ph_z = phi_slot(z);
        const R *ph_zp1 = phi_slot(z + 1);
        V4<R> *fz_rd_m = fzs + ((z - 2 + 8) & 1) * NC;   // face below plane z-1
        V4<R> *fz_rd_p = fzs + ((z - 1 + 8) & 1) * NC;   // face above plane z-1
        V4<R> *zhi_next = zhi + ((z + 1 + 8) & 1) * NC;
        // ---- phase X(z): combine plane z-1, face states of plane z --------
        static_for<0, NRX>([&](auto rc) {
            constexpr int r = decltype(rc)::value;
            constexpr int lo = r * NT, hi = (r + 1) * NT;
            const int k = t + r * NT;
            if constexpr (lo < L::X_C) {
                if (k < L::X_C) {
                    // combine plane zc = z-1 (k = t < NC)
                    if (z == z0 || !c_valid) return;
                    const int zc = z - 1;
                    const int c = cc;
                    const R phi0 = ph_zm1[c], pi0 = pf.y;
                    const V4<R> q0 = pr_zm1[c];
                    R lap_sum = R(0), gx, gy, gz;
                    {
                        const R m = ph_zm1[c - 1], p = ph_zm1[c + 1];
                        lap_sum = lap_sum + (m + p - R(2.0) * phi0);
                        gx = R(0.5) * (p - m) * P.inv_dx;
                    }
                    {
                        const R m = ph_zm1[c - PW], p = ph_zm1[c + PW];
                        lap_sum = lap_sum + (m + p - R(2.0) * phi0);
                        gy = R(0.5) * (p - m) * P.inv_dx;
                    }
                    {
                        const R m = ph_zm2[c], p = ph_z[c];
                        lap_sum = lap_sum + (m + p - R(2.0) * phi0);
                        gz = R(0.5) * (p - m) * P.inv_dx;
                    }
                    const V4<R> fxm = fxs[t + cj], fxp = fxs[t + cj + 1];
                    const V4<R> fym = fys[t], fyp = fys[t + TX];
                    const V4<R> fzm = fz_rd_m[t], fzp = fz_rd_p[t];
                    V4<R> fd;
                    if constexpr (FAST && sizeof(R) == 4) {
                        // ((dx + dy) + dz) / dx on the (x, y) and (z, w) halves
                        const float2 fa = p_mul(p_add(p_add(p_sub(lo2(fxp), lo2(fxm)), p_sub(lo2(fyp), lo2(fym))),
                                                      p_sub(lo2(fzp), lo2(fzm))),
                                                bc2(P.inv_dx));
                        const float2 fb = p_mul(p_add(p_add(p_sub(hi2(fxp), hi2(fxm)), p_sub(hi2(fyp), hi2(fym))),
                                                      p_sub(hi2(fzp), hi2(fzm))),
                                                bc2(P.inv_dx));
                        fd = v4of(fa, fb);
                    } else {
                        fd = V4<R>{R(0), R(0), R(0), R(0)};
                        fd.x = fd.x + (fxp.x - fxm.x) * P.inv_dx;
                        fd.y = fd.y + (fxp.y - fxm.y) * P.inv_dx;
                        fd.z = fd.z + (fxp.z - fxm.z) * P.inv_dx;
                        fd.w = fd.w + (fxp.w - fxm.w) * P.inv_dx;
                        fd.x = fd.x + (fyp.x - fym.x) * P.inv_dx;
                        fd.y = fd.y + (fyp.y - fym.y) * P.inv_dx;
                        fd.z = fd.z + (fyp.z - fym.z) * P.inv_dx;
                        fd.w = fd.w + (fyp.w - fym.w) * P.inv_dx;
                        fd.x = fd.x + (fzp.x - fzm.x) * P.inv_dx;
                        fd.y = fd.y + (fzp.y - fzm.y) * P.inv_dx;
                        fd.z = fd.z + (fzp.z - fzm.z) * P.inv_dx;
                        fd.w = fd.w + (fzp.w - fzm.w) * P.inv_dx;
                    }
                    const R laplacian = lap_sum * P.inv_dx * P.inv_dx;
                    const R vv = q0.x * q0.x + q0.y * q0.y + q0.z * q0.z;
                    R gam;
                    if constexpr (FAST) gam = rsqrt_approx(vmax(R(1.0) - vv, R(1e-12)));
                    else gam = R(1.0) / sqrt(vmax(R(1.0) - vv, R(1e-12)));
                    const R drag = P.eta * (gam * (pi0 + (q0.x * gx + q0.y * gy + q0.z * gz)));
                    // the thermal potential's dV/dphi at the cell's temperature, and
                    // its plasma part, exchanged like the friction
                    R dpot, src = drag;
                    if constexpr (MIXED == kThermal) {
                        const R T0 = thermal_temperature<R, FAST>(q0.w, phi0, P);
                        dpot = thermal_dpotential(phi0, T0, P);
                        src = drag + thermal_exchange(phi0, T0, P);
                    } else {
                        dpot = dpotential(phi0, P);
                    }
                    const R d_pi = laplacian - dpot - drag;
                    const R dE = -fd.x + src * pi0;
                    const R dZx = -fd.y - src * gx;
                    const R dZy = -fd.z - src * gy;
                    const R dZz = -fd.w - src * gz;
                    const size_t g = (size_t)zc * plane + c_off;
                    if constexpr (FAST && sizeof(R) == 4) {
                        // U_in + dt L and the stage combine, paired
                        const float2 dt2 = bc2(A.dt), a1 = bc2(A.a1);
                        const float2 fu = p_fma(dt2, make_float2(pi0, d_pi), make_float2(pf.x, pf.y));
                        const float2 ua = p_fma(dt2, make_float2(dE, dZx), lo2(pu));
                        const float2 ub = p_fma(dt2, make_float2(dZy, dZz), hi2(pu));
                        float2 of, oa, ob;
                        if (A.stage == 0) {
                            of = p_mul(a1, fu);
                            oa = p_mul(a1, ua);
                            ob = p_mul(a1, ub);
                        } else {
                            // rk_combine<FAST>: U^n + a1 (U1 - U^n)
                            const float2 fn = make_float2(pfn.x, pfn.y);
                            of = p_fma(a1, p_sub(fu, fn), fn);
                            oa = p_fma(a1, p_sub(ua, lo2(pun)), lo2(pun));
                            ob = p_fma(a1, p_sub(ub, hi2(pun)), hi2(pun));
                        }
                        A.field_out[g] = V2<R>{of.x, of.y};
                        A.fluid_out[g] = v4of(oa, ob);
                        return;
                    }
                    const V2<R> fu{pf.x + A.dt * pi0, pf.y + A.dt * d_pi};
                    const V4<R> uu{pu.x + A.dt * dE, pu.y + A.dt * dZx, pu.z + A.dt * dZy, pu.w + A.dt * dZz};
                    if (A.stage == 0) {
                        A.field_out[g] = V2<R>{A.a1 * fu.x, A.a1 * fu.y};
                        A.fluid_out[g] = V4<R>{A.a1 * uu.x, A.a1 * uu.y, A.a1 * uu.z, A.a1 * uu.w};
                    } else {
                        A.field_out[g] = V2<R>{rk_combine<R, FAST>(A.a0, A.a1, pfn.x, fu.x),
                                               rk_combine<R, FAST>(A.a0, A.a1, pfn.y, fu.y)};
                        A.fluid_out[g] = V4<R>{rk_combine<R, FAST>(A.a0, A.a1, pun.x, uu.x),
                                               rk_combine<R, FAST>(A.a0, A.a1, pun.y, uu.y),
                                               rk_combine<R, FAST>(A.a0, A.a1, pun.z, uu.z),
                                               rk_combine<R, FAST>(A.a0, A.a1, pun.w, uu.w)};
                    }
                    return;
                }
            }
            if (z >= z1) return;
            if constexpr (lo < L::XO_Z + L::X_Z && hi > L::XO_Z) {
                if ((lo >= L::XO_Z || k >= L::XO_Z) && k < L::XO_Z + L::X_Z) {
                    // z face states of plane z+1 (cell n)
                    const int n = k - L::XO_Z;
                    const int c = (n / TX + 2) * PW + (n % TX + 2);
                    V4<R> lo_s, hi_s;
                    face_states<R, FAST>(pr_z[c], pr_zp1[c], pr_zp2[c], P.p_floor, zmax2, lo_s, hi_s);
                    zlo[n] = lo_s;
                    zhi_next[n] = hi_s;
                    return;
                }
            }
            if constexpr (lo < L::XO_Y + L::X_Y && hi > L::XO_Y) {
                if ((lo >= L::XO_Y || k >= L::XO_Y) && k < L::XO_Y + L::X_Y) {
                    // y face states of plane z, cell row jj-1
                    const int q = k - L::XO_Y;
                    const int jj = q / TX;
                    const int c = (jj + 1) * PW + (q - jj * TX + 2);
                    V4<R> lo_s, hi_s;
                    face_states<R, FAST>(pr_z[c - PW], pr_z[c], pr_z[c + PW], P.p_floor, zmax2, lo_s, hi_s);
                    ylo[q] = lo_s;
                    yhi[q] = hi_s;
                    return;
                }
            }
            if constexpr (hi > L::XO_X) {
                if ((lo >= L::XO_X || k >= L::XO_X) && k < L::X_END) {
                    // x face states of plane z, cell column ii-1
                    const int q = k - L::XO_X;
                    const int j = q / (TX + 2);
                    const int c = (j + 2) * PW + (q - j * (TX + 2) + 1);
                    V4<R> lo_s, hi_s;
                    face_states<R, FAST>(pr_z[c - 1], pr_z[c], pr_z[c + 1], P.p_floor, zmax2, lo_s, hi_s);
                    xlo[q] = lo_s;
                    xhi[q] = hi_s;
                }
            }
        });
        if (z == z1) break;
        bool timed_out = false;
        if (z + 3 <= zlast) timed_out = !wait_plane(z + 3);
        if (__syncthreads_or(timed_out)) {
            if (t == 0) atomicOr(status, 1);
            if (tma) wait_plane(z + 3);  // bounded: drain the copy in flight
            return false;
        }
        // ---- phase Y(z): stage the next plane, primitives of z+3, fluxes ---
        if (z + 4 <= zlast) issue(z + 4);
        if (c_valid) {
            const size_t g = (size_t)z * plane + c_off;
            pf = A.field_in[g];
            pu = A.fluid_in[g];
            if (A.stage != 0) {
                pfn = A.field_n[g];
                pun = A.fluid_n[g];
            }
        }
        const bool do_a = z + 3 <= zlast;
        V4<R> *pr_a = prim_slot(z + 3);
        R *ph_a = phi_slot(z + 3);
        const V4<R> *raw_ua = raw_u + raw_slot(z + 3) * PC;
        const V2<R> *raw_fa = raw_f + raw_slot(z + 3) * PC;
        V4<R> *fz_wr = fzs + ((z + 8) & 1) * NC;
        const V4<R> *zhi_cur = zhi + ((z + 8) & 1) * NC;
        static_for<0, NRY>([&](auto rc) {
            constexpr int r = decltype(rc)::value;
            constexpr int lo = r * NT, hi = (r + 1) * NT;
            const int k = t + r * NT;
            if constexpr (lo < L::Y_A) {
                if (k < L::Y_A) {
                    const int c = ya_c[r];
                    if (!do_a || c < 0) return;
                    const V4<R> u = raw_ua[c];
                    const R phv = raw_fa[c].x;
                    ph_a[c] = phv;
                    pr_a[c] = recover_sanitised<R, FAST, MIXED>(u, P, phv, zmax2);
                    return;
                }
            }
            if constexpr (lo < L::Y_A + L::Y_Z && hi > L::Y_A) {
                if (k < L::Y_A + L::Y_Z) {
                    const int kk = k - L::Y_A;
                    R phl = R(0), phr = R(0);
                    if constexpr (MIXED == kThermal) {
                        const int c = (kk / TX + 2) * PW + (kk % TX + 2);
                        phl = ph_z[c];
                        phr = ph_zp1[c];
                    }
                    fz_wr[kk] = hll_flux<2, R, FAST, MIXED>(zhi_cur[kk], zlo[kk], zmax2, P, phl, phr);
                    return;
                }
            }
            if constexpr (lo < L::Y_A + L::Y_Z + L::Y_Y && hi > L::Y_A + L::Y_Z) {
                if (k < L::Y_A + L::Y_Z + L::Y_Y) {
                    // face between rows f-1 and f: yhi[f*TX+i] = yhi[q], ylo[(f+1)*TX+i] = ylo[q+TX]
                    const int q = k - L::Y_A - L::Y_Z;
                    R phl = R(0), phr = R(0);
                    if constexpr (MIXED == kThermal) {
                        // states of smem cells (f+1, i+2) and (f+2, i+2), f = q / TX
                        const int c = (q / TX + 1) * PW + (q % TX + 2);
                        phl = ph_z[c];
                        phr = ph_z[c + PW];
                    }
                    fys[q] = hll_flux<1, R, FAST, MIXED>(yhi[q], ylo[q + TX], zmax2, P, phl, phr);
                    return;
                }
            }
            if constexpr (hi > L::Y_A + L::Y_Z + L::Y_Y) {
                if (k < L::Y_TOTAL) {
                    // face between columns f-1 and f of row j: states j*(TX+2)+f and +1
                    const int q = k - L::Y_A - L::Y_Z - L::Y_Y;
                    const int j = q / (TX + 1);
                    R phl = R(0), phr = R(0);
                    if constexpr (MIXED == kThermal) {
                        // states of smem cells (j+2, f+1) and (j+2, f+2), f = q - j (TX+1)
                        const int c = (j + 2) * PW + (q - j * (TX + 1) + 1);
                        phl = ph_z[c];
                        phr = ph_z[c + 1];
                    }
                    fxs[q] = hll_flux<0, R, FAST, MIXED>(xhi[q + j], xlo[q + j + 1], zmax2, P, phl, phr);
                }
            }
        });
        __syncthreads();
    }
    return true;
}

template <typename R, bool FAST, int MIXED, int TY>
__global__ void __launch_bounds__(V2Layout<R, TY>::NT, V2Layout<R, TY>::MIN_BLOCKS)
    stage_v2_kernel(StageArgs<R> A, LatticeParams<R> P, int lz, const __grid_constant__ StageMaps maps,
                    int tma_ok, int *status) {
    extern __shared__ __align__(128) unsigned char smem[];
    v2_item<R, FAST, MIXED, TY>(smem, A, P, lz, &maps, tma_ok, status, blockIdx.x, blockIdx.y);
}

}  // namespace dev
}  // namespace bubble
