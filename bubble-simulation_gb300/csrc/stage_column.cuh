// Fused SSP-RK3 stage kernel, column form.
//
// The arithmetic of the reference's primitives pass and stage pass
// (shaders/primitives.wgsl:16-23, shaders/step.wgsl:92-174) with every face
// flux computed once.  A CTA owns a TX x TY column tile of the lattice (16 x
// 16, or 32 x 8 and 32 x 4) and marches it through a chunk of z planes:
//
//   * column threads, one per cell of the tile, keep their cell column's z
//     direction in registers: the primitives of three planes, the upper z
//     face state carried to the next plane, and the z fluxes above and below
//     the plane;
//   * x and y neighbours meet in shared memory: a column thread publishes
//     its recovered primitives and its cell's upper x and y face states, and
//     owns the fluxes of its cell's lower x and y faces;
//   * two halo warps recover the cross-shaped halo ring of each plane and
//     compute the face states and fluxes on the tile's far edges.
//
// Two forms of the same arithmetic (template flag LEAN):
//   * register form: the column's z pipeline (the primitives and phi of the
//     planes around z, the carried upper z face state and the lower z flux)
//     stays in registers: 83 registers, two CTAs per SM;
//   * shared form: the column thread reads its own primitives and phi back
//     from the staged rings (where they are stored anyway) and keeps the
//     carried z state and the lower z flux in per-thread shared slots: 64
//     registers, three CTAs per SM.  Each of those accesses is by the owning
//     thread, so no barrier is added.  Faster where the launch fills several
//     waves (3.1 % at 512^3), slower on small lattices that cannot fill the
//     third CTA slot.
// Both forms evaluate every value by the same operations: identical bits.
//
// Per plane z, three phases and two barriers:
//   A  recover plane z+2 (column cells into registers and shared memory,
//      halo ring into shared memory); z face states of plane z+1 and the z
//      flux z+1/2; x and y face states of plane z;
//   B  the raw plane z+4 is issued; the own-cell U_in and U^n that the
//      combine needs are loaded; x and y fluxes of plane z; z+3 is waited;
//   C  Laplacian, gradient, friction and the stage combine of plane z.
// Raw planes of U_in land in shared memory by TMA (cp.async.bulk.tensor,
// completion on an mbarrier with a bounded wait) for tiles whose halo lies
// inside the lattice, and by per-element cp.async with wrapped addresses
// elsewhere.  A chunk starts two planes early: those warm-up planes only fill
// the z pipeline, so every z face state and z flux, and every primitive
// recovery, is evaluated by the same code whatever the chunking.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"
#include "staging.cuh"
#include "tma.h"

namespace bubble {
namespace dev {

template <typename R, int TY, bool LEAN = false>
struct ColumnLayout {
    static constexpr int TX = tile_x_for(TY);
    static constexpr int PW = TX + 4, PH = TY + 4, PC = PW * PH, NC = TX * TY;
    static constexpr int NH = 64;  // halo threads: two warps
    static constexpr int NT = NC + NH;
    static constexpr int MIN_BLOCKS = sizeof(R) == 4 ? (LEAN ? 3 : 2) : 1;
    static constexpr int HR = (4 * (TX + TY) + NH - 1) / NH;  // halo cells recovered per halo thread
    static constexpr int HS = (2 * (TX + TY) + NH - 1) / NH;  // halo face states per halo thread
    static_assert(TX + TY <= NH && TY <= 32, "one halo flux per halo thread, x faces on the second warp");
    // shared memory map (bytes)
    static constexpr size_t o_rawu = 0;
    static constexpr size_t o_rawf = align128(o_rawu + 2 * PC * sizeof(V4<R>));
    static constexpr size_t o_prim = align128(o_rawf + 2 * PC * sizeof(V2<R>));
    static constexpr size_t o_phi = align128(o_prim + 3 * PC * sizeof(V4<R>));
    static constexpr size_t o_hx = align128(o_phi + 4 * PC * sizeof(R));
    static constexpr size_t o_hy = o_hx + TY * (TX + 1) * sizeof(V4<R>);
    static constexpr size_t o_lxh = o_hy + (TY + 1) * TX * sizeof(V4<R>);
    static constexpr size_t o_lyh = o_lxh + TY * sizeof(V4<R>);
    static constexpr size_t o_fx = o_lyh + TX * sizeof(V4<R>);
    static constexpr size_t o_fy = o_fx + TY * (TX + 1) * sizeof(V4<R>);
    // per halo thread: HR (cell, in-plane offset) pairs, HS (cell, stride,
    // destination, upper) quadruples, written once per item
    static constexpr size_t o_plan = align128(o_fy + (TY + 1) * TX * sizeof(V4<R>));
    // shared form: per column thread, the upper z face state it carries and
    // the flux of its lower z face
    static constexpr size_t o_hz = align128(o_plan + NH * (HR * 2 + HS * 4) * sizeof(int));
    static constexpr size_t o_fz = o_hz + (LEAN ? NC * sizeof(V4<R>) : 0);
    static constexpr size_t o_bar = o_fz + (LEAN ? NC * sizeof(V4<R>) : 0);
    static constexpr size_t bytes = o_bar + 2 * sizeof(uint64_t);
    static constexpr uint32_t plane_tx_bytes = PC * (sizeof(V4<R>) + sizeof(V2<R>));
};

// The RHS and stage combine of one cell (shaders/step.wgsl:149-173): fluxes
// of its six faces, its primitive q0 (sanitised), field values of its six
// neighbours, its own U_in (pf, pu) and U^n (pfn, pun); writes U_out at g.
template <typename R, bool FAST, int FORM>
BUBBLE_DEV void combine_cell(const StageArgs<R> &A, const LatticeParams<R> &P, uint32_t g, const V4<R> &q0, R phi0,
                             R phxm, R phxp, R phym, R phyp, R phzm, R phzp, const V4<R> &fxm, const V4<R> &fxp,
                             const V4<R> &fym, const V4<R> &fyp, const V4<R> &fzm, const V4<R> &fzp,
                             const V2<R> &pf, const V4<R> &pu, const V2<R> &pfn, const V4<R> &pun) {
    const R pi0 = pf.y;
    R lap_sum = R(0), gx, gy, gz;
    lap_sum = lap_sum + (phxm + phxp - R(2.0) * phi0);
    gx = R(0.5) * (phxp - phxm) * P.inv_dx;
    lap_sum = lap_sum + (phym + phyp - R(2.0) * phi0);
    gy = R(0.5) * (phyp - phym) * P.inv_dx;
    lap_sum = lap_sum + (phzm + phzp - R(2.0) * phi0);
    gz = R(0.5) * (phzp - phzm) * P.inv_dx;
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
    // the thermal potential's dV/dphi at the cell's temperature, and its
    // plasma part, exchanged like the friction
    R dpot, src = drag;
    if constexpr (FORM == kThermal) {
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
        A.field_out[g] = V2<R>{rk_combine<R, FAST>(A.a0, A.a1, pfn.x, fu.x), rk_combine<R, FAST>(A.a0, A.a1, pfn.y, fu.y)};
        A.fluid_out[g] = V4<R>{rk_combine<R, FAST>(A.a0, A.a1, pun.x, uu.x), rk_combine<R, FAST>(A.a0, A.a1, pun.y, uu.y),
                               rk_combine<R, FAST>(A.a0, A.a1, pun.z, uu.z), rk_combine<R, FAST>(A.a0, A.a1, pun.w, uu.w)};
    }
}

// One work item: the column tile `tile_xy` of the lattice, z chunk `chunk`
// (planes [chunk*lz, min((chunk+1)*lz, nz))), one RK stage.  Returns false
// when a bounded wait expired (bit 0 of *status is set); the CTA must then
// stop.  Usable repeatedly by one CTA: it starts with a barrier and leaves
// no copy in flight.
template <typename R, bool FAST, int FORM, int TY, bool LEAN = false>
BUBBLE_DEV bool column_item(unsigned char *smem, const StageArgs<R> &A, const LatticeParams<R> &P, int lz,
                        const StageMaps *maps, int tma_ok, int *status, int tile_xy, int chunk) {
    using L = ColumnLayout<R, TY, LEAN>;
    constexpr int TX = L::TX, NC = L::NC, NH = L::NH, PW = L::PW, PC = L::PC;
    __syncthreads();  // a previous item on this CTA is done with shared memory
    V4<R> *raw_u = reinterpret_cast<V4<R> *>(smem + L::o_rawu);
    V2<R> *raw_f = reinterpret_cast<V2<R> *>(smem + L::o_rawf);
    V4<R> *prim_s = reinterpret_cast<V4<R> *>(smem + L::o_prim);
    R *phi_s = reinterpret_cast<R *>(smem + L::o_phi);
    V4<R> *hxs = reinterpret_cast<V4<R> *>(smem + L::o_hx);   // [j][i]: upper x state of cell i-1
    V4<R> *hys = reinterpret_cast<V4<R> *>(smem + L::o_hy);   // [j][i]: upper y state of cell row j-1
    V4<R> *lxh = reinterpret_cast<V4<R> *>(smem + L::o_lxh);  // [j]: lower x state of cell xe
    V4<R> *lyh = reinterpret_cast<V4<R> *>(smem + L::o_lyh);  // [i]: lower y state of row ye
    V4<R> *fxs = reinterpret_cast<V4<R> *>(smem + L::o_fx);   // [j][i]: flux of face i-1/2
    V4<R> *fys = reinterpret_cast<V4<R> *>(smem + L::o_fy);   // [j][i]: flux of face j-1/2
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::o_bar);
    V4<R> *hz_s = reinterpret_cast<V4<R> *>(smem + L::o_hz);  // shared form: [t] carried upper z state
    V4<R> *fz_s = reinterpret_cast<V4<R> *>(smem + L::o_fz);  // shared form: [t] flux of face z-1/2

    const int t = threadIdx.x;
    const int ntx = (P.nx + TX - 1) / TX;
    const int x0 = (tile_xy % ntx) * TX;
    const int y0 = (tile_xy / ntx) * TY;
    const int z0 = chunk * lz;
    const int z1 = min(z0 + lz, P.nz);
    const int xe = min(TX, P.nx - x0);
    const int ye = min(TY, P.ny - y0);
    const R zmax2 = P.z_max * P.z_max;
    // cell indices fit 32 bits: the host rejects lattices of 2^32 cells or more
    const uint32_t plane = (uint32_t)P.nx * (uint32_t)P.ny;
    const bool tma = tma_ok && x0 >= 2 && x0 + TX + 2 <= P.nx && y0 >= 2 && y0 + TY + 2 <= P.ny;
    const int zlast = z1 + 1;  // last plane whose primitives are needed

    // Ring slots: primitives of planes z .. z+2 (3 slots), phi of planes
    // z-1 .. z+2 (4 slots), raw planes z+3, z+4 (2 slots); p >= z0 - 2.
    auto prim_slot = [&](int p) { return prim_s + ((p - z0 + 3) % 3) * PC; };
    auto phi_slot = [&](int p) { return phi_s + ((p - z0 + 4) & 3) * PC; };
    auto raw_slot = [&](int p) { return (p - z0) & 1; };

    // ---- static work plan ----------------------------------------------------
    const bool col = t < NC;
    const int ci = t % TX, cj = t / TX;
    const bool cv = col && ci < xe && cj < ye;  // a column thread with a cell
    const int cc = (cj + 2) * PW + (ci + 2);    // its cell in a staged plane
    const uint32_t c_off = (uint32_t)(y0 + cj) * (uint32_t)P.nx + (uint32_t)(x0 + ci);
    const int h = t - NC;                       // halo thread index
    // Halo plan, decoded once per item into shared memory (the halo
    // threads read their entries each plane instead of holding them in
    // registers next to the column threads' z pipeline).  Ring cells: k < 4
    // ye are the two columns on each side (cells -2, -1, xe, xe+1 of each
    // row), the rest the two rows below and above.  Face states: the upper x
    // state of cell -1 and the lower of cell xe per row, the upper y state of
    // row -1 and the lower of row ye per column.
    int2 *hr_plan = reinterpret_cast<int2 *>(smem + L::o_plan);                              // [r][h]
    int4 *hs_plan = reinterpret_cast<int4 *>(smem + L::o_plan + NH * L::HR * sizeof(int2));  // [r][h]
    if (!col) {
        static_for<0, L::HR>([&](auto rc) {
            constexpr int r = decltype(rc)::value;
            const int k = h + r * NH;
            int2 e = make_int2(-1, 0);
            if (k < 4 * (xe + ye)) {
                int i, j;
                if (k < 4 * ye) {
                    const int s = k & 3;
                    j = (k >> 2) + 2;
                    i = s < 2 ? s : xe + s;
                } else {
                    const int kk = k - 4 * ye;
                    const int row = kk / xe;
                    j = row < 2 ? row : ye + row;
                    i = kk - row * xe + 2;
                }
                e.x = j * PW + i;
                e.y = (int)((uint32_t)wrap1(y0 - 2 + j, P.ny) * (uint32_t)P.nx + (uint32_t)wrap1(x0 - 2 + i, P.nx));
            }
            hr_plan[r * NH + h] = e;
        });
        static_for<0, L::HS>([&](auto rc) {
            constexpr int r = decltype(rc)::value;
            const int k = h + r * NH;
            // (cell, stride, destination as an element index from hxs, upper)
            int4 e = make_int4(-1, 1, 0, 0);
            const int lx = (int)(L::o_lxh - L::o_hx) / (int)sizeof(V4<R>);
            const int hy = (int)(L::o_hy - L::o_hx) / (int)sizeof(V4<R>);
            const int ly = (int)(L::o_lyh - L::o_hx) / (int)sizeof(V4<R>);
            if (k < ye) e = make_int4((k + 2) * PW + 1, 1, k * (TX + 1), 1);
            else if (k < 2 * ye) e = make_int4((k - ye + 2) * PW + xe + 2, 1, lx + (k - ye), 0);
            else if (k < 2 * ye + xe) e = make_int4(PW + (k - 2 * ye) + 2, PW, hy + (k - 2 * ye), 1);
            else if (k < 2 * (xe + ye)) e = make_int4((ye + 2) * PW + (k - 2 * ye - xe) + 2, PW, ly + (k - 2 * ye - xe), 0);
            hs_plan[r * NH + h] = e;
        });
    }

    if (tma && t == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();  // publishes the mbarrier initialisation and the halo plan

    // Stage raw plane p asynchronously into its slot.
    auto issue = [&](int p) {
        const int s = raw_slot(p);
        const int gz = wrap1(p, P.nz);
        if (tma) {
            if (t == 0) {
                fence_proxy_async();
                if (A.test_tx != 0 && p == z0) {
                    // test hook: bytes that no copy delivers, and no copy issued
                    mbar_expect_tx(&bar[s], A.test_tx);
                } else {
                    mbar_expect_tx(&bar[s], L::plane_tx_bytes);
                    tma_load_4d(raw_u + s * PC, &maps->fluid, &bar[s], 0, x0 - 2, y0 - 2, gz);
                    tma_load_3d(raw_f + s * PC, &maps->field, &bar[s], 2 * (x0 - 2), y0 - 2, gz);
                }
            }
        } else {
            const uint32_t base = (uint32_t)gz * plane;
            if (cv) {
                cp_async_v4(raw_u + s * PC + cc, A.fluid_in + (base + c_off));
                cp_async_v2(raw_f + s * PC + cc, A.field_in + (base + c_off));
            }
            if (!col) {
                static_for<0, L::HR>([&](auto rc) {
                    constexpr int r = decltype(rc)::value;
                    const int2 e = hr_plan[r * NH + h];
                    if (e.x >= 0) {
                        cp_async_v4(raw_u + s * PC + e.x, A.fluid_in + (base + (uint32_t)e.y));
                        cp_async_v2(raw_f + s * PC + e.x, A.field_in + (base + (uint32_t)e.y));
                    }
                });
            }
            cp_async_commit();
        }
    };
    // Wait for raw plane p (`newer`: plane p+1 was issued after it); false
    // when the bounded wait expired.
    auto wait_raw = [&](int p, bool newer) -> bool {
        if (tma) return mbar_wait_bounded(&bar[raw_slot(p)], ((p - z0) >> 1) & 1, A.wait_shift);
        if (newer) cp_async_wait_but_one();
        else cp_async_wait_all();
        return true;
    };
    // On expiry: record it, wait (bounded) for the copies in flight, stop.
    auto give_up = [&](int p, bool newer) {
        if (t == 0) atomicOr(status, 1);
        if (tma) {
            wait_raw(p, false);
            if (newer) wait_raw(p + 1, false);
        }
    };

    issue(z0);
    issue(z0 + 1);  // zlast >= z0 + 2

    // The z pipeline of a column (register form): q0, q1 = primitives of
    // planes z, z+1; ph_m .. ph1 = phi of planes z-1 .. z+1; hiz = upper z
    // state of cell z; fz_m = flux of face z-1/2.  The shared form reads the
    // same values from the rings and from hz_s / fz_s.  The warm-up planes
    // z0-2, z0-1 come straight from global memory.
    V4<R> q0{R(0), R(0), R(0), R(0)}, q1 = q0, hiz = q0, fz_m = q0;
    R ph_m = R(0), ph0 = R(0), ph1 = R(0);
    if (cv) {
        const uint32_t ga = (uint32_t)wrap1(z0 - 2, P.nz) * plane + c_off;
        const uint32_t gb = (uint32_t)wrap1(z0 - 1, P.nz) * plane + c_off;
        const V4<R> ua = A.fluid_in[ga], ub = A.fluid_in[gb];
        const R pa = A.field_in[ga].x, pb = A.field_in[gb].x;
        const V4<R> qa = recover_sanitised<R, FAST, FORM>(ua, P, pa, zmax2);
        const V4<R> qb = recover_sanitised<R, FAST, FORM>(ub, P, pb, zmax2);
        if constexpr (LEAN) {
            prim_slot(z0 - 2)[cc] = qa;
            prim_slot(z0 - 1)[cc] = qb;
            phi_slot(z0 - 2)[cc] = pa;
            phi_slot(z0 - 1)[cc] = pb;
            hz_s[t] = V4<R>{R(0), R(0), R(0), R(0)};
        } else {
            q0 = qa;
            q1 = qb;
            ph0 = pa;
            ph1 = pb;
        }
    }
    {
        const bool to = !wait_raw(z0, true);
        if (__syncthreads_or(to)) {
            give_up(z0, true);
            return false;
        }
    }

    for (int z = z0 - 2; z < z1; ++z) {
        const bool act = z >= z0;  // planes below z0 only fill the z pipeline
        const V4<R> *pr_z = prim_slot(z);
        const R *ph_z = phi_slot(z);
        // ---- phase A ---------------------------------------------------------
        V4<R> q2{R(0), R(0), R(0), R(0)};
        R ph2 = R(0);
        {
            const int s = raw_slot(z + 2);
            const V4<R> *ru = raw_u + s * PC;
            const V2<R> *rf = raw_f + s * PC;
            V4<R> *pw = prim_slot(z + 2);
            R *fw = phi_slot(z + 2);
            if (cv) {
                const V4<R> u = ru[cc];
                ph2 = rf[cc].x;
                q2 = recover_sanitised<R, FAST, FORM>(u, P, ph2, zmax2);
                pw[cc] = q2;
                fw[cc] = ph2;
            }
            if (!col) {
                static_for<0, L::HR>([&](auto rc) {
                    constexpr int r = decltype(rc)::value;
                    const int c = hr_plan[r * NH + h].x;
                    if (c >= 0) {
                        const V4<R> u = ru[c];
                        const R phv = rf[c].x;
                        fw[c] = phv;
                        pw[c] = recover_sanitised<R, FAST, FORM>(u, P, phv, zmax2);
                    }
                });
            }
        }
        V4<R> fz_p{R(0), R(0), R(0), R(0)}, lox, loy;
        if (cv) {
            // z face states of cell z+1 and the flux of face z+1/2
            V4<R> c0 = q0, c1 = q1;
            if constexpr (LEAN) {
                c0 = pr_z[cc];
                c1 = prim_slot(z + 1)[cc];
            }
            V4<R> lo1, hi1;
            face_states<R, FAST>(c0, c1, q2, P.p_floor, zmax2, lo1, hi1);
            if constexpr (LEAN) {
                if (z >= z0 - 1)
                    fz_p = hll_flux<2, R, FAST, FORM>(hz_s[t], lo1, zmax2, P, ph_z[cc], phi_slot(z + 1)[cc]);
                hz_s[t] = hi1;
            } else {
                if (z >= z0 - 1) fz_p = hll_flux<2, R, FAST, FORM>(hiz, lo1, zmax2, P, ph0, ph1);
                hiz = hi1;
            }
            if (act) {
                V4<R> hix, hiy;
                face_states<R, FAST>(pr_z[cc - 1], c0, pr_z[cc + 1], P.p_floor, zmax2, lox, hix);
                hxs[cj * (TX + 1) + ci + 1] = hix;
                face_states<R, FAST>(pr_z[cc - PW], c0, pr_z[cc + PW], P.p_floor, zmax2, loy, hiy);
                hys[(cj + 1) * TX + ci] = hiy;
            }
        }
        if (act && !col) {
            static_for<0, L::HS>([&](auto rc) {
                constexpr int r = decltype(rc)::value;
                const int4 e = hs_plan[r * NH + h];
                if (e.x >= 0) {
                    V4<R> lo_s, hi_s;
                    face_states<R, FAST>(pr_z[e.x - e.y], pr_z[e.x], pr_z[e.x + e.y], P.p_floor, zmax2, lo_s, hi_s);
                    hxs[e.z] = e.w ? hi_s : lo_s;
                }
            });
        }
        __syncthreads();
        // ---- phase B ---------------------------------------------------------
        if (z + 4 <= zlast) issue(z + 4);
        // own-cell U_in and U^n of the combine: loaded a phase ahead in the
        // register form; at the combine in the shared form, where twelve
        // registers held across the barrier made the 64-register build
        // recompute its uniform address arithmetic per thread (integer
        // instructions 154 -> 85 per cell, 512^3 step 11.01 -> 10.92 ms)
        V2<R> pf{R(0), R(0)}, pfn{R(0), R(0)};
        V4<R> pu{R(0), R(0), R(0), R(0)}, pun{R(0), R(0), R(0), R(0)};
        if (act) {
            if (cv) {
                if constexpr (!LEAN) {
                    const uint32_t g = (uint32_t)z * plane + c_off;
                    pf = A.field_in[g];
                    pu = A.fluid_in[g];
                    if (A.stage != 0) {
                        pfn = A.field_n[g];
                        pun = A.fluid_n[g];
                    }
                }
                R phl_x = R(0), phl_y = R(0);
                if constexpr (FORM == kThermal) {
                    phl_x = ph_z[cc - 1];
                    phl_y = ph_z[cc - PW];
                }
                R phc = ph0;
                if constexpr (LEAN) phc = ph_z[cc];
                fxs[cj * (TX + 1) + ci] = hll_flux<0, R, FAST, FORM>(hxs[cj * (TX + 1) + ci], lox, zmax2, P, phl_x, phc);
                fys[cj * TX + ci] = hll_flux<1, R, FAST, FORM>(hys[cj * TX + ci], loy, zmax2, P, phl_y, phc);
            } else if (!col) {
                if (h < 32) {
                    // y face above row ye-1, column h
                    if (h < xe) {
                        R phl = R(0), phr = R(0);
                        if constexpr (FORM == kThermal) {
                            phl = ph_z[(ye + 1) * PW + h + 2];
                            phr = ph_z[(ye + 2) * PW + h + 2];
                        }
                        fys[ye * TX + h] = hll_flux<1, R, FAST, FORM>(hys[ye * TX + h], lyh[h], zmax2, P, phl, phr);
                    }
                } else if (h - 32 < ye) {
                    // x face right of column xe-1, row h-32
                    const int j = h - 32;
                    R phl = R(0), phr = R(0);
                    if constexpr (FORM == kThermal) {
                        phl = ph_z[(j + 2) * PW + xe + 1];
                        phr = ph_z[(j + 2) * PW + xe + 2];
                    }
                    fxs[j * (TX + 1) + xe] = hll_flux<0, R, FAST, FORM>(hxs[j * (TX + 1) + xe], lxh[j], zmax2, P, phl, phr);
                }
            }
        }
        bool timed_out = false;
        if (z + 3 <= zlast) timed_out = !wait_raw(z + 3, z + 4 <= zlast);
        if (__syncthreads_or(timed_out)) {
            give_up(z + 3, z + 4 <= zlast);
            return false;
        }
        // ---- phase C: combine plane z ------------------------------------------
        if constexpr (LEAN) {
            if (act && cv) {
                const uint32_t g = (uint32_t)z * plane + c_off;
                pf = A.field_in[g];
                pu = A.fluid_in[g];
                if (A.stage != 0) {
                    pfn = A.field_n[g];
                    pun = A.fluid_n[g];
                }
                combine_cell<R, FAST, FORM>(A, P, (uint32_t)z * plane + c_off, pr_z[cc], ph_z[cc], ph_z[cc - 1],
                                            ph_z[cc + 1], ph_z[cc - PW], ph_z[cc + PW], phi_slot(z - 1)[cc],
                                            phi_slot(z + 1)[cc], fxs[cj * (TX + 1) + ci],
                                            fxs[cj * (TX + 1) + ci + 1], fys[cj * TX + ci], fys[(cj + 1) * TX + ci],
                                            fz_s[t], fz_p, pf, pu, pfn, pun);
            }
            if (cv) fz_s[t] = fz_p;
        } else {
            if (act && cv) {
                combine_cell<R, FAST, FORM>(A, P, (uint32_t)z * plane + c_off, q0, ph0, ph_z[cc - 1], ph_z[cc + 1],
                                            ph_z[cc - PW], ph_z[cc + PW], ph_m, ph1, fxs[cj * (TX + 1) + ci],
                                            fxs[cj * (TX + 1) + ci + 1], fys[cj * TX + ci], fys[(cj + 1) * TX + ci],
                                            fz_m, fz_p, pf, pu, pfn, pun);
            }
            q0 = q1;
            q1 = q2;
            ph_m = ph0;
            ph0 = ph1;
            ph1 = ph2;
            fz_m = fz_p;
        }
    }
    return true;
}

template <typename R, bool FAST, int FORM, int TY, bool LEAN>
__global__ void __launch_bounds__(ColumnLayout<R, TY, LEAN>::NT, ColumnLayout<R, TY, LEAN>::MIN_BLOCKS)
    stage_kernel(StageArgs<R> A, LatticeParams<R> P, int lz, const __grid_constant__ StageMaps maps,
                    int tma_ok, int *status) {
    extern __shared__ __align__(128) unsigned char smem[];
    column_item<R, FAST, FORM, TY, LEAN>(smem, A, P, lz, &maps, tma_ok, status, blockIdx.x, blockIdx.y);
}

}  // namespace dev
}  // namespace bubble
