// k_isspa.cu -- IS-SPA solvent kernels for sm_103a.
//
// Replaces the reference's three-kernel IS-SPA pass (src/isspa_force_cuda.cu:
// 73-107 MC points, :110-206 field, :208-327 force) with two kernels:
//
//  field:  one thread-column per MC point.  The point is generated in the
//          prologue from Philox counters (no stored RNG state), every atom of
//          the point's window is streamed through shared memory, and the
//          density product, in-range count, mean field and far field are
//          reduced in registers and combined across the S warps that split the
//          atom loop in a fixed order.  One writer per point: no atomics, no
//          racy re-read of the density (the reference's atomicMul, :195).
//          The per-point prologue of the reference's force kernel (|E|, unit
//          field, Langevin averages, 1/n; :253-273) is computed here once per
//          point instead of once per (atom, point) pair.
//  force:  one thread per receiving atom (or two); work items are (window,
//          128-atom tile, point chunk), and each item streams its points
//          through shared memory in stages of 128 (broadcast reads); per-thread
//          FP32 partial sums are flushed once per stage into int64 fixed-point
//          registers and once per item into the atom's accumulator, so the
//          final force is independent of scheduling order.
#include <algorithm>
#include <cuda_runtime.h>

#include <type_traits>

#include "kernels.h"
#include "md_device.cuh"
#include "philox.h"

namespace isspa {

namespace {

constexpr int kFieldThreads = 128;
constexpr int kForceThreads = 128;

// <P1>, <P2>, <P3> of a Langevin dipole in a field of magnitude x.  Below 5
// the ratios i_l/i_(l-1) of modified spherical Bessel functions are taken from
// their backward continued fraction r_l = x / (2l+1 + x r_(l+1)) (all terms
// positive, no cancellation); above, the closed forms of the reference
// (isspa_force_cuda.cu:270-273, 283, 287) are exact to float rounding.
__device__ __forceinline__ void langevin3(float x, float &p1, float &p2, float &p3) {
    if (x < 5.0f) {
        float r = 0.0f, r2 = 0.0f, r3 = 0.0f;
#pragma unroll
        for (int l = 12; l >= 1; --l) {
            r = __fdiv_rn(x, (float)(2 * l + 1) + x * r);
            if (l == 3) r3 = r;
            if (l == 2) r2 = r;
        }
        p1 = r;
        p2 = r * r2;
        p3 = p2 * r3;
    } else {
        const float c = 1.0f / tanhf(x);
        const float ix = 1.0f / x;
        const float ix2 = ix * ix;
        p1 = c - ix;
        p2 = 1.0f + 3.0f * ix2 - 3.0f * c * ix;
        p3 = (1.0f + 15.0f * ix2) * c - 6.0f * ix - 15.0f * ix2 * ix;
    }
}

// MC point p (index within its window) of `owner` at position xa with radius
// rm: uniform in the ball r^2 < 0.99 (isspa_force_cuda.cu:92-100).
__device__ __forceinline__ void mc_point(uint32_t p, uint32_t window, uint32_t step, uint32_t k0,
                                         uint32_t k1, float4 xa, float rm, float &px, float &py,
                                         float &pz) {
    float mx = 0.5f, my = 0.0f, mz = 0.0f;
    for (uint32_t att = 0; att < 64u; ++att) {
        u32x4 o = philox4x32_10(u32x4{p, att, step, (window << 8) | 0u}, k0, k1);
        float x = __fmaf_rn(2.0f, u01(o.x), -1.0f);
        float y = __fmaf_rn(2.0f, u01(o.y), -1.0f);
        float z = __fmaf_rn(2.0f, u01(o.z), -1.0f);
        if (dist2f(x, y, z) < 0.99f) {
            mx = x; my = y; mz = z;
            break;
        }
    }
    px = __fmaf_rn(mx, rm, xa.x);
    py = __fmaf_rn(my, rm, xa.y);
    pz = __fmaf_rn(mz, rm, xa.z);
}

// 1-D bulk copies (cp.async.bulk, the TMA engine's untiled form) from global
// into this CTA's shared memory, completed on an mbarrier; every wait is
// bounded.  Both addresses are 16-byte aligned and sizes multiples of 16.
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// Waits for phase `parity` of the barrier with non-blocking polls; false once
// kBulkWaitNs of global time have passed (a deadline in time, not in polls).
constexpr unsigned long long kBulkWaitNs = 1000000000ull;
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
    const unsigned long long t0 = global_ns();
    for (;;) {
        unsigned done;
        asm volatile(
            "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > kBulkWaitNs) return false;
        __nanosleep(32);
    }
}

// One MC point's records side by side in shared memory: a single base address
// per point, the five float4 at immediate offsets (q3 / q4 picked per lane).
struct alignas(16) PointRec {
    float4 q[5];
};

// Block shape of the field kernel: S warps split the atom loop of each group
// of 32 points; 4 warps per block up to S = 4, then 32*S threads.
template <int S>
struct FieldShape {
    static constexpr int kThreads = S >= 4 ? 32 * S : kFieldThreads;  // kThreads/(32 S) point groups
};

// VOTE: the atom loop takes groups of four atoms and one warp vote per group
// (see below); same operations in the same order as the per-pair loop.
// TMA: the window's atoms arrive in rounds of 128 by 1-D bulk copies of the
// position array, double-buffered behind two mbarriers (thread 0 issues round
// r + 2 as soon as round r has been read); e0 q and the table row are formed
// at use (the same products, so the same results).  One warp vote per round
// makes a bounded wait that gave up block-uniform: the block then flags
// kStatusTimeout, waits (bounded) for its copies still in flight and exits.
// FUSE: the tile's point records are also left in s_rec[slot] for a force
// phase of the same block (which follows a barrier after this function; no
// barrier of this function comes after a thread's early return).
template <int S, bool GEN, bool RAW, bool VOTE, bool TMA = false, bool FUSE = false>
__device__ __forceinline__ void field_tile(const FieldArgs &a, int tile_index, PointRec *s_rec = nullptr) {
    static_assert(!FUSE || (GEN && !RAW && !TMA), "the fused pass draws its points and stages by loads");
    constexpr int kT = FieldShape<S>::kThreads;
    // atoms staged per round: four per thread below a split of 4, so the
    // warps' compute phases between barriers are four times longer (64 windows
    // at split 1: 1.779 against 1.808 ms per launch; at split 8 one per thread
    // measured faster); a multiple of S either way, so each warp still visits
    // its atoms (j = sp mod S) in increasing order, whatever the round length
    constexpr int kA = TMA ? 128 : (S >= 4 ? kT : 4 * kT);
    __shared__ alignas(16) float4 s_atom[TMA ? 2 : 1][kA];
    __shared__ int s_row[TMA ? 1 : kA];
    __shared__ alignas(8) unsigned long long s_bar[2];
    __shared__ float s_red[S > 1 ? 8 : 1][kT];
    constexpr bool kShareDraws = GEN && S >= 4;
    __shared__ float s_pt[3][kShareDraws ? kT / S : 1];  // the block's points, drawn once

    const int4 tile = a.tiles[tile_index];
    const WinDev W = a.win[tile.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = warp / S, sp = warp % S;
    const int slot = grp * 32 + lane;
    const bool valid = slot < tile.z;
    const long long pg = tile.y + (valid ? slot : tile.z - 1);  // global point
    const long long pw = pg - W.point_off;                        // point within window
    const int owner = W.atom_off + (int)(pw / a.n_mc);
    const float4 xo = a.pos[owner];
    const float rm = __ldg(a.rmax + a.atype[owner].y);
    const float rm2 = __fmul_rn(rm, rm);
    const float L = W.box, h = W.hbox;

    const int nb = a.n_gbins;
    const int n_rounds = (W.n_atoms + kA - 1) / kA;
    // one round of the window's atoms into shared memory: [j0, j0 + jn)
    auto stage_round = [&](int j0, int jn) {
        auto stage = [&](int i) {
            const int j = W.atom_off + j0 + i;
            float4 xj = a.pos[j];
            xj.w = a.e0 * xj.w;  // e0*q (isspa_force_cuda.cu:179, :183)
            s_atom[0][i] = xj;
            s_row[i] = a.atype[j].y * nb;
        };
        if (kA == kT) {
            if (threadIdx.x < jn) stage(threadIdx.x);
        } else {
#pragma unroll 1
            for (int i = threadIdx.x; i < jn; i += kT) stage(i);
        }
    };
    auto issue_round = [&](int r) {  // TMA, thread 0
        const int jn = min(kA, W.n_atoms - r * kA);
        bulk_load(s_atom[r & 1], a.pos + W.atom_off + r * kA, 16u * (unsigned)jn, &s_bar[r & 1]);
    };
    // the first round is staged (or issued) before the points are known, so
    // its loads overlap the draws and the barrier below covers both
    if (TMA) {
        if (threadIdx.x == 0) {
            mbar_init(&s_bar[0]);
            mbar_init(&s_bar[1]);
            mbar_init_fence();
            issue_round(0);
            if (n_rounds > 1) issue_round(1);
        }
    } else {
        stage_round(0, min(kA, W.n_atoms));
    }

    float px, py, pz;
    if (kShareDraws) {
        // one warp of each group draws the group's 32 points (rejection
        // sampling, divergent attempt counts); the other S-1 warps wait at the
        // barrier instead of repeating the draws on issue slots the SM needs
        // (1100 atoms, S = 8: 0.0876 against 0.0925 ms per launch; with S = 2
        // the barrier costs more than the one repeated draw saves)
        if (sp == 0) {
            mc_point((uint32_t)pw, (uint32_t)tile.x, *a.step_ptr, a.seed_lo, a.seed_hi, xo, rm, px, py, pz);
            s_pt[0][slot] = px;
            s_pt[1][slot] = py;
            s_pt[2][slot] = pz;
        }
        __syncthreads();
        px = s_pt[0][slot];
        py = s_pt[1][slot];
        pz = s_pt[2][slot];
    } else {
        if (GEN) {
            mc_point((uint32_t)pw, (uint32_t)tile.x, *a.step_ptr, a.seed_lo, a.seed_hi, xo, rm, px, py, pz);
        } else {
            px = a.pts_in[3 * pg + 0];
            py = a.pts_in[3 * pg + 1];
            pz = a.pts_in[3 * pg + 2];
        }
        __syncthreads();  // first round staged
    }

    float w = 1.0f;
    int n = 0;
    float ex = 0.f, ey = 0.f, ez = 0.f, fx = 0.f, fy = 0.f, fz = 0.f;
    const float g_r0 = a.g_r0, g_dr = a.g_dr, g_inv = a.g_inv;
    const float e_r0 = a.e_r0, e_dr = a.e_dr, e_inv = a.e_inv;
    // the field table shares the density bin (:170-174): interpolation across
    // that bin's edges is continuous only when both tables use one radial grid
    const bool one_grid = g_r0 == e_r0 && g_dr == e_dr;

    // geometry of the pair (point, staged atom k); true when inside rmax of
    // the owner's type (:154)
    int buf = 0, jbase = 0;  // staged buffer and first atom of the current round
    auto geom = [&](int k, float &rx, float &ry, float &rz, float &c) {
        const float4 xj = s_atom[TMA ? buf : 0][k];
        rx = mimg(px - xj.x, L, h);
        ry = mimg(py - xj.y, L, h);
        rz = mimg(pz - xj.z, L, h);
        const float d2 = dist2f(rx, ry, rz);
        const float ri = rsqrtf(d2);
        c = (TMA ? a.e0 * xj.w : xj.w) * (ri * ri * ri);
        return d2 <= rm2;
    };
    // ex.. accumulates the in-range contributions (Coulomb and tabulated
    // field), fx.. the out-of-range Coulomb field E0; E = ex.. + fx..  d2 and
    // ri are recomputed from the same operands (same values) to keep fewer
    // registers live across a group.
    auto accum = [&](int k, float rx, float ry, float rz, float c) {
        const float d2 = dist2f(rx, ry, rz);
        if (d2 <= rm2) {
            const float ri = rsqrtf(d2);
            ++n;
            ex = fmaf(-c, rx, ex);
            ey = fmaf(-c, ry, ey);
            ez = fmaf(-c, rz, ez);
            const float dist = one_grid ? density_table_dist(d2, ri) : __fsqrt_rn(d2);
            const int bin = (int)__fmul_rn(__fsub_rn(dist, g_r0), g_inv);
            if (bin < 0) {
                w = 0.0f;
            } else if (bin < nb) {
                const int row = TMA ? __ldg(&a.atype[W.atom_off + jbase + k].y) * nb : s_row[k];
                const float4 t = __ldg(a.gtab + row + bin);
                const float fg = (dist - fmaf((float)bin, g_dr, g_r0)) * g_inv;
                w *= fmaf(fg, t.y - t.x, t.x);
                const float fe = (dist - fmaf((float)bin, e_dr, e_r0)) * e_inv;
                const float et = fmaf(fe, t.w - t.z, t.z) * ri;
                ex = fmaf(et, rx, ex);
                ey = fmaf(et, ry, ey);
                ez = fmaf(et, rz, ez);
            }
        } else {
            fx = fmaf(-c, rx, fx);
            fy = fmaf(-c, ry, fy);
            fz = fmaf(-c, rz, fz);
        }
    };

    for (int j0 = 0, r = 0; j0 < W.n_atoms; j0 += kA, ++r) {
        const int jn = min(kA, W.n_atoms - j0);
        if (TMA) {
            buf = r & 1;
            jbase = j0;
            if (r > 0) {
                __syncthreads();  // round r - 1 has been read: its buffer takes round r + 1
                if (threadIdx.x == 0 && r + 1 < n_rounds) {
                    proxy_fence();
                    issue_round(r + 1);
                }
            }
            if (!__syncthreads_and(mbar_wait(&s_bar[buf], (unsigned)(r >> 1) & 1u))) {
                if (threadIdx.x == 0) {
                    atomicOr(a.status, kStatusTimeout);
                    for (int q = r; q < min(r + 2, n_rounds); ++q) mbar_wait(&s_bar[q & 1], (unsigned)(q >> 1) & 1u);
                }
                return;
            }
        } else if (j0 > 0) {
            __syncthreads();  // the previous round has been read
            stage_round(j0, jn);
            __syncthreads();
        }
        int k = sp;
        // Groups of kG staged atoms: one warp vote tells whether any lane has
        // any of them inside rmax.  When none does, their out-of-range Coulomb
        // terms are summed without per-pair branches; the accumulators see the
        // same operations in the same order either way.  It pays where few
        // groups have an atom in range (large systems: 16 384 atoms in a
        // 120 A box, 21.5 against 23.4 ms per launch) and costs registers
        // where many do (1100 atoms: 0.092 against 0.087 ms), so the
        // autotuner chooses.
        constexpr int kG = 4;
        for (; VOTE && k + (kG - 1) * S < jn; k += kG * S) {
            float rx[kG], ry[kG], rz[kG], c[kG];
            bool any = false;
#pragma unroll
            for (int u = 0; u < kG; ++u) any = geom(k + u * S, rx[u], ry[u], rz[u], c[u]) || any;
            if (__any_sync(0xffffffffu, any)) {
#pragma unroll
                for (int u = 0; u < kG; ++u) accum(k + u * S, rx[u], ry[u], rz[u], c[u]);
            } else {
#pragma unroll
                for (int u = 0; u < kG; ++u) {
                    fx = fmaf(-c[u], rx[u], fx);
                    fy = fmaf(-c[u], ry[u], fy);
                    fz = fmaf(-c[u], rz[u], fz);
                }
            }
        }
        if (VOTE) {
#pragma unroll 1
            for (; k < jn; k += S) {  // at most kG - 1 atoms
                float rx, ry, rz, c;
                geom(k, rx, ry, rz, c);
                accum(k, rx, ry, rz, c);
            }
        } else {
#pragma unroll 4
            for (; k < jn; k += S) {
                float rx, ry, rz, c;
                geom(k, rx, ry, rz, c);
                accum(k, rx, ry, rz, c);
            }
        }
    }

    if (S > 1) {
        s_red[0][threadIdx.x] = w;
        s_red[1][threadIdx.x] = __int_as_float(n);
        s_red[2][threadIdx.x] = ex;
        s_red[3][threadIdx.x] = ey;
        s_red[4][threadIdx.x] = ez;
        s_red[5][threadIdx.x] = fx;
        s_red[6][threadIdx.x] = fy;
        s_red[7][threadIdx.x] = fz;
        __syncthreads();
        if (sp != 0) return;
#pragma unroll
        for (int s = 1; s < S; ++s) {
            const int o = (grp * S + s) * 32 + lane;
            w *= s_red[0][o];
            n += __float_as_int(s_red[1][o]);
            ex += s_red[2][o];
            ey += s_red[3][o];
            ez += s_red[4][o];
            fx += s_red[5][o];
            fy += s_red[6][o];
            fz += s_red[7][o];
        }
    }
    if (!valid) return;
    ex += fx;  // total mean field = in-range part + out-of-range Coulomb part
    ey += fy;
    ez += fz;

    if (RAW) {
        a.raw_e[pg] = make_float4(ex, ey, ez, w);
        a.raw_e0[pg] = make_float4(fx, fy, fz, (float)n);
    }
    if (n <= 0) {  // cannot happen: the owner itself is always in range
        atomicOr(a.status, kStatusBounds);
        n = 1;
        w = 0.0f;
    }
    const float inv_n = 1.0f / (float)n;
    const float sden = w * inv_n;
    const float mag = __fsqrt_rn(dist2f(ex, ey, ez));
    const float im = mag > 0.0f ? 1.0f / mag : 0.0f;
    float p1, p2, p3;
    langevin3(mag, p1, p2, p3);
    // term masks act here: a zero amplitude or far dipole removes a term exactly
    const bool mp = a.terms & 1, cdd = a.terms & 4;
    const float a1 = mp ? kP0 * p1 * sden : 0.0f;
    const float a2 = mp ? kQ0 * p2 * sden : 0.0f;
    const float a3 = mp ? kO0 * p3 * sden : 0.0f;
    const float hx = ex * im, hy = ey * im, hz = ez * im;
    const float cd = cdd ? kP0 * inv_n * (1.0f / 3.0f) : 0.0f;  // p0 E0 / (3 n)
    const float4 r0 = make_float4(px, py, pz, sden);
    const float4 r1 = make_float4(hx, hy, hz, 1.5f * a2);
    const float4 r2 = make_float4(7.5f * a2, 17.5f * a3, 3.0f * a2, 7.5f * a3);
    const float4 r3 = make_float4(a1 * hx, a1 * hy, a1 * hz, 1.5f * a3);
    const float4 r4 = make_float4(fmaf(a1, hx, cd * fx), fmaf(a1, hy, cd * fy), fmaf(a1, hz, cd * fz), 1.5f * a3);
    a.out.q0[pg] = r0;
    a.out.q1[pg] = r1;
    a.out.q2[pg] = r2;
    a.out.q3[pg] = r3;
    a.out.q4[pg] = r4;
    if (FUSE) {
        s_rec[slot].q[0] = r0;
        s_rec[slot].q[1] = r1;
        s_rec[slot].q[2] = r2;
        s_rec[slot].q[3] = r3;
        s_rec[slot].q[4] = r4;
    }
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned int *p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <int S, bool GEN, bool RAW, bool VOTE, bool TMA = false>
__global__ void __launch_bounds__(FieldShape<S>::kThreads) field_kernel(FieldArgs a) {
    pdl_wait();
    pdl_trigger();
    // the stamp is read before the tile's work (kept in shared memory), so the
    // block's exit does not wait on it
    __shared__ unsigned int s_stamp;
    if (a.tile_flag && threadIdx.x == 0) s_stamp = *a.ov_epoch + 1u;
    field_tile<S, GEN, RAW, VOTE, TMA>(a, blockIdx.x);
    if (a.tile_flag) {
        // the tile's records are written: the barrier orders every thread's
        // stores before thread 0's release, which the force items acquire
        __syncthreads();
        if (threadIdx.x == 0) st_release_u32(a.tile_flag + blockIdx.x, s_stamp);
    }
}

// LJ = include the tabulated mean LJ force (term bit 2); the multipole and CDD
// terms are shaped by the per-point constants of the field pass.  A = receiving
// atoms per thread (t and t + 128/A of the item): each staged point's records
// are read once from shared memory for A atoms.  Every atom sees the same
// arithmetic in the same order whatever A is.
template <int A>
struct ForceShape {
    static constexpr int kThreads = kForceThreads / A;
    static constexpr int kMinBlocks = A == 1 ? 10 : 12;  // 48 / 85 registers per thread
};

// One MC point's force terms on a receiving atom, r = point - atom (minimum
// image) and d2 = |r|^2: the multipole terms (:274-289, with the CDD term
// (:306-312) folded into the record D) into q per unit -q_i vtot_i, the
// tabulated mean LJ force (:291-305) into l per unit -vtot_i.  rm2 and frow
// belong to the atom's type; FAR: the point is known to lie outside rmax.
template <bool LJ, bool FAR>
__device__ __forceinline__ void point_force(const float4 *R, float rx, float ry, float rz, float d2, float rm2,
                                            int frow, const ForceArgs &a, float &qx, float &qy, float &qz,
                                            float &lx, float &ly, float &lz) {
    const float4 E = R[1];
    const float4 K = R[2];
    const bool inside = !FAR && d2 <= rm2;  // (:291)
    const float ri = rsqrtf(d2);
    const float ri2 = ri * ri;
    const float ri3 = ri2 * ri;
    const float ri5 = ri3 * ri2;
    const float4 D = R[inside ? 3 : 4];
    const float w = fmaf(E.x, rx, fmaf(E.y, ry, E.z * rz));
    const float dD = fmaf(D.x, rx, fmaf(D.y, ry, D.z * rz));
    const float g = w * ri2;
    float X = (w * g) * fmaf(K.y, g, K.x);
    X = fmaf(3.0f, dD, X) - E.w;
    X = fmaf(-K.w, g, X);
    const float cR = X * ri5;
    const float cE = fmaf(-D.w, ri2, fmaf(K.w, g, K.z) * g) * ri3;
    qx = fmaf(cR, rx, fmaf(-cE, E.x, fmaf(-ri3, D.x, qx)));
    qy = fmaf(cR, ry, fmaf(-cE, E.y, fmaf(-ri3, D.y, qy)));
    qz = fmaf(cR, rz, fmaf(-cE, E.z, fmaf(-ri3, D.z, qz)));
    if (LJ && inside) {
        const float dist = __fsqrt_rn(d2);
        const int bin = (int)__fmaf_rn(__fsub_rn(dist, a.f_r0), a.f_inv, 0.5f);
        if (bin >= 0 && bin < a.n_f) {
            const float2 tv = __ldg(a.ftab + frow + bin);
            const float fr = (dist - fmaf((float)bin, a.f_dr, a.f_r0)) * a.f_inv;
            const float fv = fmaf(fr, tv.y - tv.x, tv.x) * R[0].w * ri;
            lx = fmaf(fv, rx, lx);
            ly = fmaf(fv, ry, ly);
            lz = fmaf(fv, rz, lz);
        }
    }
}

// VOTE (one atom per thread only): points in groups of four with one warp
// vote per group on "any lane has any of them inside rmax"; a group with none
// takes the out-of-range records without the per-pair select and tabulated-LJ
// branch.  Same operations in the same order as the per-pair loop.  It keeps
// four points' geometry live (64 registers, 8 blocks per SM).
template <bool LJ, int A, bool VOTE = false>
__device__ __forceinline__ void force_item(const ForceArgs &a, int item_index) {
    static_assert(!VOTE || A == 1, "the voted loop takes one receiving atom per thread");
    constexpr int kT = ForceShape<A>::kThreads;
    __shared__ PointRec s_p[kForceThreads];
    const int4 item = a.items[item_index];
    const WinDev W = a.win[item.x];
    const int2 ch = a.chunks[item.w];
    const int t = threadIdx.x;
    const float L = W.box, h = W.hbox;
    const int nf = a.n_f;
    bool active[A];
    int ai[A], frow[A];
    float4 xi[A];
    float rm2[A], vt[A];
#pragma unroll
    for (int u = 0; u < A; ++u) {
        active[u] = t + u * kT < item.z;
        ai[u] = item.y + (active[u] ? t + u * kT : 0);
        xi[u] = a.pos[ai[u]];
        const int ity = a.atype[ai[u]].y;
        const float rm = __ldg(a.rmax + ity);
        rm2[u] = __fmul_rn(rm, rm);
        frow[u] = ity * nf;
        vt[u] = __ldg(a.vtot + ity);
    }
    // Per-stage FP32 partial sums (at most kForceThreads points) are folded into
    // per-thread fixed-point registers, so FP32 rounding never spans more than
    // one stage; one set of atomics per atom and work item.
    long long fxa[A], fya[A], fza[A];
#pragma unroll
    for (int u = 0; u < A; ++u) fxa[u] = fya[u] = fza[u] = 0;

    for (int p0 = 0; p0 < ch.y; p0 += kForceThreads) {
        float qx[A], qy[A], qz[A];  // polarisation terms, per unit -q_i vtot_i
        float lx[A], ly[A], lz[A];  // tabulated LJ, per unit -vtot_i
#pragma unroll
        for (int u = 0; u < A; ++u) qx[u] = qy[u] = qz[u] = lx[u] = ly[u] = lz[u] = 0.f;
        const int pn = min(kForceThreads, ch.y - p0);
        __syncthreads();
        for (int i = t; i < pn; i += kT) {
            const long long pg = (long long)ch.x + p0 + i;
            // through L2: in the single-kernel step the records were written
            // by other blocks of the same launch
            s_p[i].q[0] = __ldcg(a.pts.q0 + pg);
            s_p[i].q[1] = __ldcg(a.pts.q1 + pg);
            s_p[i].q[2] = __ldcg(a.pts.q2 + pg);
            s_p[i].q[3] = __ldcg(a.pts.q3 + pg);
            s_p[i].q[4] = __ldcg(a.pts.q4 + pg);
        }
        __syncthreads();
        // the pair (staged point k, receiving atom u) after its geometry; FAR:
        // the point is known to lie outside rmax of the atom's type
        auto pair = [&](int k, int u, float rx, float ry, float rz, float d2, auto far) {
            point_force<LJ, decltype(far)::value>(s_p[k].q, rx, ry, rz, d2, rm2[u], frow[u], a, qx[u], qy[u], qz[u],
                                                  lx[u], ly[u], lz[u]);
        };
        int k = 0;
        if (VOTE) {
            for (; k + 3 < pn; k += 4) {
                float rx[4], ry[4], rz[4], d2[4];
                bool any = false;
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const float4 P = s_p[k + v].q[0];
                    rx[v] = mimg(P.x - xi[0].x, L, h);
                    ry[v] = mimg(P.y - xi[0].y, L, h);
                    rz[v] = mimg(P.z - xi[0].z, L, h);
                    d2[v] = dist2f(rx[v], ry[v], rz[v]);
                    any = any || d2[v] <= rm2[0];
                }
                if (__any_sync(0xffffffffu, any)) {
#pragma unroll
                    for (int v = 0; v < 4; ++v) pair(k + v, 0, rx[v], ry[v], rz[v], d2[v], std::false_type{});
                } else {
#pragma unroll
                    for (int v = 0; v < 4; ++v) pair(k + v, 0, rx[v], ry[v], rz[v], d2[v], std::true_type{});
                }
            }
        }
#pragma unroll 4
        for (; k < pn; ++k) {
            const float4 P = s_p[k].q[0];
#pragma unroll
            for (int u = 0; u < A; ++u) {
                const float rx = mimg(P.x - xi[u].x, L, h);
                const float ry = mimg(P.y - xi[u].y, L, h);
                const float rz = mimg(P.z - xi[u].z, L, h);
                pair(k, u, rx, ry, rz, dist2f(rx, ry, rz), std::false_type{});
            }
        }
#pragma unroll
        for (int u = 0; u < A; ++u) {
            const float Fx = -vt[u] * fmaf(xi[u].w, qx[u], lx[u]);
            const float Fy = -vt[u] * fmaf(xi[u].w, qy[u], ly[u]);
            const float Fz = -vt[u] * fmaf(xi[u].w, qz[u], lz[u]);
            if (active[u]) check_force(a.status, Fx, Fy, Fz);
            fxa[u] += to_fix(Fx);
            fya[u] += to_fix(Fy);
            fza[u] += to_fix(Fz);
        }
    }
#pragma unroll
    for (int u = 0; u < A; ++u) {
        if (!active[u]) continue;
        unsigned long long *acc = a.facc + 3 * (long long)ai[u];
        atomicAdd(acc + 0, (unsigned long long)fxa[u]);
        atomicAdd(acc + 1, (unsigned long long)fya[u]);
        atomicAdd(acc + 2, (unsigned long long)fza[u]);
    }
}

// Overlap mode: thread 0 waits until every field tile that holds a point of
// this item's chunk carries the current stamp (the wait gives up after
// kOverlapWaitNs of global time: kStatusTimeout, and the item adds nothing).
// Deadlock-free under a programmatic launch, whose blocks are scheduled only
// once every field block has started; after an ordinary launch the stamps
// are all in place.
constexpr unsigned long long kOverlapWaitNs = 500000000ull;
__device__ __forceinline__ bool wait_item_tiles(const ForceArgs &a, int item_index) {
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        const int4 item = a.items[item_index];
        const WinDev W = a.win[item.x];
        const int2 ch = a.chunks[item.w];
        const unsigned int stamp = *a.ov_epoch + 1u;
        const long long q0 = (long long)ch.x - W.point_off, q1 = q0 + ch.y - 1;
        const int base = a.tile_base[item.x];
        const int t1 = base + (int)(q1 / a.tile_pts);
        int ok = 1;
        const unsigned long long t_start = global_ns();
        for (int tt = base + (int)(q0 / a.tile_pts); ok && tt <= t1; ++tt)
            while (ld_acquire_u32(a.tile_flag + tt) != stamp) {
                if (global_ns() - t_start > kOverlapWaitNs) {
                    atomicOr(a.status, kStatusTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(128);
            }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}
template <bool LJ, int A, bool VOTE = false>
__global__ void __launch_bounds__(ForceShape<A>::kThreads, VOTE ? 8 : ForceShape<A>::kMinBlocks)
    force_kernel(ForceArgs a) {
    if (!a.overlap) pdl_wait();
    pdl_trigger();
    if (!a.overlap || wait_item_tiles(a, blockIdx.x)) force_item<LJ, A, VOTE>(a, blockIdx.x);
}

// Forces of a field tile's own np points (records in shared memory) on every
// atom of its window.  Threads take (atom, point group) pairs: G groups of
// consecutive points, G = min(np, threads / atoms) (at least 1), so small
// windows keep the block's threads busy; each pair runs the force pass's
// per-pair arithmetic and sums its group in FP32.  The groups' fixed-point
// values meet in shared memory (s_acc, windows of up to kFusedSmemAtoms
// atoms), so the block adds one set of global atomics per atom: every block
// of a small window adds into the same few hundred words, and per-group
// global atomics queued on them.
constexpr int kFusedSmemAtoms = 512;
template <bool LJ>
__device__ __forceinline__ void tile_point_forces(const ForceArgs &a, const WinDev &W, const PointRec *s_rec,
                                                  int np, unsigned long long *s_acc) {
    const bool smem = W.n_atoms <= kFusedSmemAtoms;
    const float L = W.box, h = W.hbox;
    const int n = W.n_atoms;
    const int G = max(1, min(np, (int)blockDim.x / max(n, 1)));
    const int per = (np + G - 1) / G;
    for (int idx = threadIdx.x; idx < n * G; idx += blockDim.x) {
        const int i = idx % n, grp = idx / n;
        const int k0 = grp * per, k1 = min(np, k0 + per);
        const int ai = W.atom_off + i;
        const float4 xi = a.pos[ai];
        const int ity = a.atype[ai].y;
        const float rm = __ldg(a.rmax + ity);
        const float rm2 = __fmul_rn(rm, rm);
        const int frow = ity * a.n_f;
        const float vt = __ldg(a.vtot + ity);
        float qx = 0.f, qy = 0.f, qz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
#pragma unroll 4
        for (int k = k0; k < k1; ++k) {
            const float4 P = s_rec[k].q[0];
            const float rx = mimg(P.x - xi.x, L, h);
            const float ry = mimg(P.y - xi.y, L, h);
            const float rz = mimg(P.z - xi.z, L, h);
            point_force<LJ, false>(s_rec[k].q, rx, ry, rz, dist2f(rx, ry, rz), rm2, frow, a, qx, qy, qz, lx, ly, lz);
        }
        if (k1 <= k0) continue;
        const float Fx = -vt * fmaf(xi.w, qx, lx);
        const float Fy = -vt * fmaf(xi.w, qy, ly);
        const float Fz = -vt * fmaf(xi.w, qz, lz);
        check_force(a.status, Fx, Fy, Fz);
        unsigned long long *acc = smem ? s_acc + 3 * i : a.facc + 3 * (long long)ai;
        atomicAdd(acc + 0, (unsigned long long)to_fix(Fx));
        atomicAdd(acc + 1, (unsigned long long)to_fix(Fy));
        atomicAdd(acc + 2, (unsigned long long)to_fix(Fz));
    }
    if (!smem) return;
    __syncthreads();
    for (int c = threadIdx.x; c < 3 * n; c += blockDim.x) atomicAdd(a.facc + 3 * (long long)W.atom_off + c, s_acc[c]);
}

// Field and force passes fused for small windows: each block computes its
// tile's points (the field kernel's code, records also kept in shared
// memory), then those points' forces on every atom of the window.  A point's
// force on an atom needs only that point's record, so no other block's result
// is waited for; one launch per step instead of two, and no record round trip
// through L2.  Forces equal the separate passes' up to FP32 summation order
// (sums over a tile's points instead of a force work item's).
template <int S, bool VOTE>
__global__ void __launch_bounds__(FieldShape<S>::kThreads) field_force_kernel(FieldArgs f, ForceArgs g) {
    pdl_wait();
    pdl_trigger();
    __shared__ PointRec s_rec[FieldShape<S>::kThreads / S];
    __shared__ unsigned long long s_acc[3 * kFusedSmemAtoms];
    for (int c = threadIdx.x; c < 3 * kFusedSmemAtoms; c += blockDim.x) s_acc[c] = 0ull;
    field_tile<S, true, false, VOTE, false, true>(f, blockIdx.x, s_rec);  // (its first barrier orders s_acc)
    __syncthreads();
    const int4 tile = f.tiles[blockIdx.x];
    tile_point_forces<true>(g, f.win[tile.x], s_rec, tile.z, s_acc);
}

// The whole MD step in one cooperative launch, for engines whose step is
// latency-bound (a few thousand atoms or fewer): every kernel of a step would
// otherwise pay its own launch, ramp-up and drain.  Phase 1: field tiles
// (split 4), nonbond items, bonded terms and the restraint COMs (none of them
// needs another's result); grid barrier; phase 2: force items; grid barrier;
// phase 3: restraint forces and leapfrog per atom, step counter.  Each phase
// runs the separate kernels' per-item code, so for the same work lists the
// trajectory is bit-identical to theirs.  Both barriers are bounded (the
// fused integrator's); a barrier that gives up flags kStatusTimeout and the
// step integrates nothing.
template <bool NB_ALL>
__global__ void __launch_bounds__(kFieldThreads, 4) step_kernel(StepArgs a) {
    extern __shared__ float2 s_ab[];
    const uint32_t step = *a.integ.lf.step_ptr;
    if (a.nonbond.n_items > 0) stage_ljab(a.nonbond, s_ab);
    // field tiles and nonbond items as one list over the blocks, so a block
    // left without a tile takes a nonbond item instead of queueing behind one
    const int n1 = a.field.n_tiles + a.nonbond.n_items;
    for (int t = blockIdx.x; t < n1; t += gridDim.x) {
        if (t < a.field.n_tiles) field_tile<4, true, false, false>(a.field, t);
        else nonbond_item<true, NB_ALL>(a.nonbond, t - a.field.n_tiles, s_ab);
    }
    bonded_terms(a.integ.bonded);
    restraint_coms(a.integ);
    if (!grid_barrier(a.integ.bar, a.integ.lf.status)) return;
    for (int t = blockIdx.x; t < a.force.n_items; t += gridDim.x) force_item<true, 1, false>(a.force, t);
    if (!grid_barrier(a.integ.bar, a.integ.lf.status)) return;
    integrate_atoms(a.integ, step);
}

template <int S, bool GEN, bool RAW, bool VOTE = false, bool TMA = false>
void launch_field_t(const FieldArgs &a, cudaStream_t s) {
    launch_chain(field_kernel<S, GEN, RAW, VOTE, TMA>, a.n_tiles, FieldShape<S>::kThreads, s, a);
}

template <int S>
void launch_field_s(const FieldArgs &a, bool raw, cudaStream_t s) {
    const bool gen = a.pts_in == nullptr;
    // the vote and TMA variants give the same results; the raw-field captures
    // (tests, adjoint) always take the per-pair loop with plain staging
    if (a.tma && gen && !raw) {
        if (a.vote) launch_field_t<S, true, false, true, true>(a, s);
        else launch_field_t<S, true, false, false, true>(a, s);
    } else if (a.vote && !raw) {
        if (gen) launch_field_t<S, true, false, true>(a, s);
        else launch_field_t<S, false, false, true>(a, s);
    } else if (gen && !raw) launch_field_t<S, true, false>(a, s);
    else if (gen && raw) launch_field_t<S, true, true>(a, s);
    else if (!gen && !raw) launch_field_t<S, false, false>(a, s);
    else launch_field_t<S, false, true>(a, s);
}

template <int S>
int field_bps() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, field_kernel<S, true, false, false>, FieldShape<S>::kThreads, 0);
    return n;
}

}  // namespace

int field_block_threads() { return kFieldThreads; }
int force_block_threads() { return kForceThreads; }

void launch_field(const FieldArgs &a, int split, bool raw, cudaStream_t s) {
    if (a.n_tiles <= 0) return;
    switch (split) {
        case 16: launch_field_s<16>(a, raw, s); break;
        case 8: launch_field_s<8>(a, raw, s); break;
        case 4: launch_field_s<4>(a, raw, s); break;
        case 2: launch_field_s<2>(a, raw, s); break;
        default: launch_field_s<1>(a, raw, s); break;
    }
}

int field_points_per_block(int split) { return split >= 4 ? 32 : 128 / split; }

int field_blocks_per_sm(int split) {
    switch (split) {
        case 16: return field_bps<16>();
        case 8: return field_bps<8>();
        case 4: return field_bps<4>();
        case 2: return field_bps<2>();
        default: return field_bps<1>();
    }
}

int force_blocks_per_sm(int atoms_per_thread) {
    int n = 0;
    if (atoms_per_thread == 2)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, force_kernel<true, 2>, ForceShape<2>::kThreads, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, force_kernel<true, 1>, ForceShape<1>::kThreads, 0);
    return n;
}

int step_threads() { return kFieldThreads; }

int step_max_blocks(int n_lj_types) {
    int dev = 0, sms = 0, per_a = 0, per_b = 0;
    const size_t smem = sizeof(float2) * (size_t)std::max(1, n_lj_types * n_lj_types);
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_a, step_kernel<true>, kFieldThreads, smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_b, step_kernel<false>, kFieldThreads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return sms * std::min(per_a, per_b);
}

cudaError_t launch_step(const StepArgs &a, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kFieldThreads);
    cfg.dynamicSmemBytes = sizeof(float2) * (size_t)std::max(1, a.nonbond.n_lj_types * a.nonbond.n_lj_types);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (a.nonbond.terms == 7) return cudaLaunchKernelEx(&cfg, step_kernel<true>, a);
    return cudaLaunchKernelEx(&cfg, step_kernel<false>, a);
}

bool field_force_fusable(int split) { return split == 4 || split == 8 || split == 16; }

void launch_field_force(const FieldArgs &f, const ForceArgs &g, int split, cudaStream_t s) {
    if (f.n_tiles <= 0) return;
    const bool v = f.vote != 0;
    switch (split) {
        case 16:
            if (v) launch_chain(field_force_kernel<16, true>, f.n_tiles, FieldShape<16>::kThreads, s, f, g);
            else launch_chain(field_force_kernel<16, false>, f.n_tiles, FieldShape<16>::kThreads, s, f, g);
            break;
        case 8:
            if (v) launch_chain(field_force_kernel<8, true>, f.n_tiles, FieldShape<8>::kThreads, s, f, g);
            else launch_chain(field_force_kernel<8, false>, f.n_tiles, FieldShape<8>::kThreads, s, f, g);
            break;
        default:
            if (v) launch_chain(field_force_kernel<4, true>, f.n_tiles, FieldShape<4>::kThreads, s, f, g);
            else launch_chain(field_force_kernel<4, false>, f.n_tiles, FieldShape<4>::kThreads, s, f, g);
            break;
    }
}

void launch_force(const ForceArgs &a, cudaStream_t s) {
    if (a.n_items <= 0) return;
    if (a.vote && a.atoms_per_thread != 2) {
        if (a.terms & 2) launch_chain(force_kernel<true, 1, true>, a.n_items, ForceShape<1>::kThreads, s, a);
        else launch_chain(force_kernel<false, 1, true>, a.n_items, ForceShape<1>::kThreads, s, a);
    } else if (a.atoms_per_thread == 2) {
        if (a.terms & 2) launch_chain(force_kernel<true, 2>, a.n_items, ForceShape<2>::kThreads, s, a);
        else launch_chain(force_kernel<false, 2>, a.n_items, ForceShape<2>::kThreads, s, a);
    } else {
        if (a.terms & 2) launch_chain(force_kernel<true, 1>, a.n_items, ForceShape<1>::kThreads, s, a);
        else launch_chain(force_kernel<false, 1>, a.n_items, ForceShape<1>::kThreads, s, a);
    }
}

}  // namespace isspa
