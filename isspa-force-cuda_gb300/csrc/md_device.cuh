// md_device.cuh -- device code of the pair, bonded, umbrella and integrator
// passes, shared by their own kernels (k_md.cu) and the single-kernel step
// (k_isspa.cu).  Everything here runs per work item or per thread; the
// kernels decide the grid.
#pragma once
#include <climits>
#include <cuda_runtime.h>
#include <type_traits>

#include "kernels.h"
#include "philox.h"

namespace isspa {
namespace {

constexpr int kNbThreads = 128;
constexpr int kNbMaxAB = 4096;  // LJ type pairs held in shared memory (up to 64 LJ types)

// One work item: 128 receiving atoms i (one per thread) against nj partners j
// starting at item.w, streamed through shared memory in stages of 128.  The
// per-stage FP32 sums are folded into fixed point per stage, and stages start
// at multiples of 128 partners from the window's first atom whatever the item
// length, so the forces do not depend on the partners per item (an autotuned
// shape).  Exclusions and the self pair are found per stage as a 128-bit mask
// from the atom's sorted exclusion list; a group of 32 partners that no lane
// of the warp excludes runs without per-pair checks.  SMEM_AB: the LJ (A, B)
// table of every ordered type pair sits in shared memory (dynamic, nt^2
// float2) instead of a global gather per pair.  ALL: every term on (mask 7).
template <bool SMEM_AB, bool ALL>
__device__ __forceinline__ void nonbond_item(const NonbondArgs &a, int item_index, const float2 *s_ab) {
    __shared__ float4 s_x[kNbThreads];
    __shared__ float4 s_c[kNbThreads];  // rmax_j, (2 rmax_j)^2, 8 rmax_j, (1-1/ep)/(24 rmax_j^4)
    __shared__ int s_t[kNbThreads];
    const int4 item = a.items[item_index];
    const int nj = a.items_nj[item_index];
    const WinDev W = a.win[item.x];
    const int t = threadIdx.x;
    const bool active = t < item.z;
    const int i = item.y + (active ? t : 0);
    const float4 xi = a.pos[i];
    const int nt = a.n_lj_types;
    const int trow = a.atype[i].x * nt;
    const float L = W.box, h = W.hbox;
    const int terms = ALL ? 7 : a.terms;
    const float epf = 1.0f - 1.0f / kEp;
    const float kfar = -2.0f * epf / 3.0f;

    // exclusion cursor: first entry >= first partner of this item; the list
    // is sorted, so an item outside [first, last] entry needs no walk
    const int end = a.excl_start[i + 1];
    int cur = a.excl_start[i];
    if (cur < end) {
        if (a.excl[end - 1] < item.w || a.excl[cur] >= item.w + nj) cur = end;
        else
            while (cur < end && a.excl[cur] < item.w) ++cur;
    }

    long long fxa = 0, fya = 0, fza = 0;  // per-stage partial sums in fixed point
    for (int j0 = 0; j0 < nj; j0 += kNbThreads) {
        const int jn = min(kNbThreads, nj - j0);
        const int jb = item.w + j0;  // first partner of the stage
        // exclusion / self bits of this stage's 128 partners
        unsigned m[4] = {0u, 0u, 0u, 0u};  // register-resident: constant indices only
        auto set_bit = [&](int b) {
            const unsigned bit = 1u << (b & 31);
#pragma unroll
            for (int q = 0; q < 4; ++q) m[q] |= (b >> 5) == q ? bit : 0u;
        };
        for (; cur < end; ++cur) {
            const int b = a.excl[cur] - jb;
            if (b >= kNbThreads || j0 + b >= nj) break;
            set_bit(b);
        }
        if (i - jb >= 0 && i - jb < kNbThreads) set_bit(i - jb);
        float ax = 0.f, ay = 0.f, az = 0.f;
        __syncthreads();
        if (t < jn) {
            const int j = jb + t;
            s_x[t] = a.pos[j];
            const int2 ty = a.atype[j];
            const float rm = __ldg(a.rmax + ty.y);
            const float two = 2.0f * rm;
            const float r2 = rm * rm;
            s_c[t] = make_float4(rm, __fmul_rn(two, two), 8.0f * rm, epf / (24.0f * r2 * r2));
            s_t[t] = ty.x;
        }
        __syncthreads();
        // the pair (i, staged partner k); EX: excluded (IS-SPA correction
        // only).  MASKED: the exclusion bit and the self pair are applied by
        // selects instead of branches (the self pair gets d2 = 1 and adds
        // nothing), so a group with exclusions keeps an unrolled loop; the
        // values are those of the branching form.
        auto pair_t = [&](int k, bool ex, bool self, auto masked) {
            constexpr bool MASKED = decltype(masked)::value;
            const float4 xj = s_x[k];
            const float rx = mimg(xi.x - xj.x, L, h);
            const float ry = mimg(xi.y - xj.y, L, h);
            const float rz = mimg(xi.z - xj.z, L, h);
            const float d2 = MASKED && self ? 1.0f : dist2f(rx, ry, rz);
            const float ri = rsqrtf(d2);
            const float ri2 = ri * ri;
            const float qq = xi.w * xj.w;
            float fs = 0.0f;
            if (terms & 4) {  // IS-SPA long-range dielectric correction (:141-147)
                const float4 c = s_c[k];
                fs = d2 > c.y ? kfar * qq * ri2 * ri : -qq * c.w * (c.z - 3.0f * d2 * ri);
            }
            if (MASKED || !ex) {
                float fp = fs;
                if (terms & 1) {  // LJ (:131-132)
                    const float2 ab = SMEM_AB ? s_ab[trow + s_t[k]] : __ldg(a.ljab + trow + s_t[k]);
                    const float r6 = ri2 * ri2 * ri2;
                    fp += r6 * fmaf(12.0f * ab.x, r6, -6.0f * ab.y) * ri2;
                }
                if (terms & 2) fp += qq * ri2 * ri;  // Coulomb (:136)
                fs = MASKED && ex ? fs : fp;
            }
            if (MASKED) fs = self ? 0.0f : fs;
            ax = fmaf(fs, rx, ax);
            ay = fmaf(fs, ry, ay);
            az = fmaf(fs, rz, az);
        };
        auto pair = [&](int k, bool ex) { pair_t(k, ex, false, std::false_type{}); };
#pragma unroll
        for (int q = 0; q < kNbThreads / 32; ++q) {
            const int k0 = 32 * q;
            if (k0 >= jn) break;
            const int kn = min(32, jn - k0);
            const unsigned mq = m[q];
            if (__any_sync(0xffffffffu, mq != 0u)) {
                // exclusions or the self pair in this group: masked pairs,
                // unrolled like the unmasked group below
                const int self_k = i - (jb + k0);  // the self pair's k, if in this group
                if (kn == 32) {
#pragma unroll 4
                    for (int k = 0; k < 32; ++k)
                        pair_t(k0 + k, (mq >> k) & 1u, k == self_k, std::true_type{});
                } else {
#pragma unroll 1
                    for (int k = 0; k < kn; ++k)
                        pair_t(k0 + k, (mq >> k) & 1u, k == self_k, std::true_type{});
                }
            } else if (kn == 32) {
#pragma unroll 8
                for (int k = 0; k < 32; ++k) pair(k0 + k, false);
            } else {
#pragma unroll 1
                for (int k = 0; k < kn; ++k) pair(k0 + k, false);
            }
        }
        if (active) check_force(a.status, ax, ay, az);
        fxa += to_fix(ax);
        fya += to_fix(ay);
        fza += to_fix(az);
    }
    if (!active) return;
    unsigned long long *acc = a.facc + 3 * (long long)i;
    atomicAdd(acc + 0, (unsigned long long)fxa);
    atomicAdd(acc + 1, (unsigned long long)fya);
    atomicAdd(acc + 2, (unsigned long long)fza);
}

// Stages the LJ (A, B) table of every ordered type pair into shared memory
// (read only after the item's first barrier).
__device__ __forceinline__ void stage_ljab(const NonbondArgs &a, float2 *s_ab) {
    for (int k = threadIdx.x; k < a.n_lj_types * a.n_lj_types; k += blockDim.x) s_ab[k] = a.ljab[k];
}

// Bonded terms in FP32.  Image vectors as the reference decides them
// (min_image), then formulations that stay well conditioned where the
// reference's closed forms cancel:
//   * bond:     f = 2k (r0 - |r|) / |r| r, the difference taken before the
//               division (bond_force_cuda.cu:36-50 writes 2k (r0/|r| - 1));
//   * angle:    theta = atan2(|r1 x r2|, -r1.r2) and the force directions as
//               triple products, r1 x (r1 x r2) / c11 = (c12/c11) r1 - r2 and
//               r2 x (r1 x r2) / c22 = r1 - (c12/c22) r2, over |r1 x r2| =
//               sqrt(c11 c22 - c12^2) (angle_force_cuda.cu:19-52);
//   * dihedral: the torsion gradient of Blondel & Karplus, J. Comput. Chem. 17
//               (1996) 1132, with phi = atan2 of the cross-product sine and
//               cosine: no acos and no 1/sin(phi), so near-planar torsions keep
//               FP32 accuracy.  The reference's energy is V (1 + cos(n phi_u -
//               phase)) with the unsigned angle phi_u = acos(cos phi) in [0, pi]
//               (dih_force_cuda.cu:86-135), so dU/dphi = -V n sin(n |phi| -
//               phase) sgn(phi); an exactly planar torsion gets no force, as
//               the reference's |cos phi| >= 1 branch.
// Every term adds its forces through to_fix into the int64 accumulator, so
// the result does not depend on the order of the atomics and the fused
// integrator (which runs the same term functions) reproduces it bit for bit.
struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 rvec(const float4 *pos, int p, int q, float L, float h) {
    const float4 a = pos[p], b = pos[q];
    return F3{mimg(a.x - b.x, L, h), mimg(a.y - b.y, L, h), mimg(a.z - b.z, L, h)};
}
__device__ __forceinline__ float dotf(F3 a, F3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ F3 crossf(F3 a, F3 b) {
    return F3{fmaf(a.y, b.z, -a.z * b.y), fmaf(a.z, b.x, -a.x * b.z), fmaf(a.x, b.y, -a.y * b.x)};
}
__device__ __forceinline__ F3 scalef(float s, F3 a) { return F3{s * a.x, s * a.y, s * a.z}; }

// Double-float values (hi + lo, two FP32 words) from the error-free
// transformations of Knuth (TwoSum) and Dekker (TwoProduct, here with an FMA):
// the bond stretch r0 - |r| and the angle bend theta - theta0 of a geometry
// near its minimum are small differences of O(1) quantities, which FP32 alone
// resolves only to ~1e-7 absolute (a relative error of the force that grows
// as the force vanishes).  Carried in double-float they keep ~1e-7 of their
// own size; every operation is an FP32 instruction (__fadd_rn / __fmul_rn /
// fmaf, never contracted or reassociated).
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return DF{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const DF s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const DF p = two_prod(a.hi, b.hi);
    return fast_two_sum(p.hi, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo)));
}
// a.b of float vectors, and |a|, in double-float
__device__ __forceinline__ DF df_dot(F3 a, F3 b) {
    return df_add(df_add(two_prod(a.x, b.x), two_prod(a.y, b.y)), two_prod(a.z, b.z));
}
__device__ __forceinline__ DF df_sqrt(DF a) {  // a > 0; one Newton step on the FP32 root
    const float s = __fsqrt_rn(a.hi);
    const float res = __fadd_rn(fmaf(-s, s, a.hi), a.lo);
    return fast_two_sum(s, __fdiv_rn(res, __fmul_rn(2.0f, s)));
}
__device__ __forceinline__ float df_float(DF a) { return __fadd_rn(a.hi, a.lo); }


// Fixed-point scatter of one atom's share of a term.
struct FixAdd {
    unsigned long long *facc;
    int *status;
    __device__ __forceinline__ void operator()(int atom, F3 f) const {
        check_force(status, f.x, f.y, f.z);
        fix_add3(facc + 3 * (long long)atom, f.x, f.y, f.z);
    }
};

// Term idx of the concatenated (enabled) bond, angle and dihedral lists.
template <class Add>
__device__ __forceinline__ void bonded_term(const BondedArgs &a, long long idx, const Add &add) {
    const long long nb = a.do_bonds ? a.n_bonds : 0;
    const long long na = a.do_angles ? a.n_angles : 0;
    const long long nd = a.do_dihs ? a.n_dihs : 0;
    if (idx < nb) {  // bond_force_cuda.cu:36-50
        const int4 b = a.bonds[idx];
        const WinDev W = a.win[a.atom_win[b.x]];
        const F3 r = rvec(a.pos, b.x, b.y, W.box, W.hbox);
        const float2 p = a.bond_par[b.z];
        const DF d = df_sqrt(df_dot(r, r));
        const float stretch = df_float(df_add(two_sum(p.y, -d.hi), DF{-d.lo, 0.0f}));  // r0 - |r|
        const float f = __fdiv_rn(__fmul_rn(p.x, stretch), df_float(d));
        add(b.x, scalef(f, r));
        add(b.y, scalef(-f, r));
        return;
    }
    idx -= nb;
    if (idx < na) {  // angle_force_cuda.cu:19-52
        const int4 g = a.angles[idx];
        const WinDev W = a.win[a.atom_win[g.x]];
        const F3 r1 = rvec(a.pos, g.x, g.y, W.box, W.hbox);
        const F3 r2 = rvec(a.pos, g.y, g.z, W.box, W.hbox);
        // |r1 x r2| and r1.r2 in double-float, then theta - theta0 as the angle
        // of (-r1.r2, |r1 x r2|) rotated by -theta0 (cos and sin of theta0
        // given in double-float per angle type)
        const DF wx = df_add(two_prod(r1.y, r2.z), df_neg(two_prod(r1.z, r2.y)));
        const DF wy = df_add(two_prod(r1.z, r2.x), df_neg(two_prod(r1.x, r2.z)));
        const DF wz = df_add(two_prod(r1.x, r2.y), df_neg(two_prod(r1.y, r2.x)));
        const DF s2 = df_add(df_add(df_mul(wx, wx), df_mul(wy, wy)), df_mul(wz, wz));
        if (!(s2.hi > 0.0f)) return;  // collinear: the reference's 1/0
        const DF s = df_sqrt(s2);
        const DF c12 = df_dot(r1, r2);
        const float4 cs = a.angle_cs[g.w];  // cos theta0 (hi, lo), sin theta0 (hi, lo)
        const DF ct{cs.x, cs.y}, st{cs.z, cs.w};
        const float y = df_float(df_add(df_mul(s, ct), df_mul(c12, st)));
        const float x = fmaf(s.hi, st.hi, -__fmul_rn(c12.hi, ct.hi));
        const float bend = atan2f(y, x);  // theta - theta0
        const float2 p = a.angle_par[g.w];
        const F3 w{wx.hi, wy.hi, wz.hi};
        const float f = __fdiv_rn(__fmul_rn(p.x, bend), df_float(s));
        const F3 fi = scalef(__fdiv_rn(f, dotf(r1, r1)), crossf(r1, w));
        const F3 fk = scalef(__fdiv_rn(f, dotf(r2, r2)), crossf(r2, w));
        add(g.x, fi);
        add(g.y, F3{-(fi.x + fk.x), -(fi.y + fk.y), -(fi.z + fk.z)});
        add(g.z, fk);
        return;
    }
    idx -= na;
    if (idx < nd) {  // dih_force_cuda.cu:48-135
        const int4 d = a.dihs[idx];  // absolute atom indices
        const int raw = a.dih_type[idx];
        const int ty = raw & 0x3FFFFFFF;
        const WinDev W = a.win[a.atom_win[d.x]];
        const float L = W.box, h = W.hbox;
        if (raw & 0x40000000) {  // scaled 1-4 when atoms.z > 0 && atoms.w > 0 (:60-82)
            const float2 ab = __ldg(a.ljab + a.atype[d.x].x * a.n_lj_types + a.atype[d.w].x);
            const float2 sc = a.sc14[ty];
            const F3 r14 = rvec(a.pos, d.x, d.w, L, h);
            const float rm = dotf(r14, r14);
            const float ri2 = __frcp_rn(rm);
            const float r6 = ri2 * ri2 * ri2;
            const float fe = __fdiv_rn(a.pos[d.x].w * a.pos[d.w].w, rm * __fsqrt_rn(rm) * sc.x);
            const float fv = __fdiv_rn(r6 * fmaf(12.0f * ab.x, r6, -6.0f * ab.y) * ri2, sc.y);
            const float f = fe + fv;
            add(d.x, scalef(f, r14));
            add(d.w, scalef(-f, r14));
        }
        // Blondel-Karplus: F = x1 - x2, G = x2 - x3, H = x4 - x3
        const F3 F = rvec(a.pos, d.x, d.y, L, h);
        const F3 G = rvec(a.pos, d.y, d.z, L, h);
        const F3 Hm = rvec(a.pos, d.z, d.w, L, h);  // x3 - x4 = -H
        const F3 H{-Hm.x, -Hm.y, -Hm.z};
        const F3 A = crossf(F, G), B = crossf(H, G);
        const float A2 = dotf(A, A), B2 = dotf(B, B);
        const float Gn = __fsqrt_rn(dotf(G, G));
        if (!(A2 > 0.0f) || !(B2 > 0.0f) || !(Gn > 0.0f)) return;  // collinear triple
        const float cphi = dotf(A, B);
        const float sphi = __fdiv_rn(dotf(crossf(B, A), G), Gn);
        if (sphi == 0.0f) return;  // exactly planar: |cos phi| = 1 in the reference
        const float phi_u = atan2f(fabsf(sphi), cphi);
        const float4 p = a.dih_par[ty];
        // -dU/dphi (signed phi)
        const float g = p.x * p.y * sinf(fmaf(p.x, phi_u, -p.z)) * (sphi > 0.0f ? 1.0f : -1.0f);
        const float FG = dotf(F, G), HG = dotf(H, G);
        const float ga = __fdiv_rn(g * Gn, A2);   // force on x1 = -g Gn / A2 A ...
        const float gb = __fdiv_rn(g * Gn, B2);
        const float fa = __fdiv_rn(g * FG, A2 * Gn);
        const float fb = __fdiv_rn(g * HG, B2 * Gn);
        const F3 f1 = scalef(-ga, A);
        const F3 f4 = scalef(gb, B);
        const F3 f2{fmaf(ga + fa, A.x, -fb * B.x), fmaf(ga + fa, A.y, -fb * B.y), fmaf(ga + fa, A.z, -fb * B.z)};
        const F3 f3{fmaf(fb - gb, B.x, -fa * A.x), fmaf(fb - gb, B.y, -fa * A.y), fmaf(fb - gb, B.z, -fa * A.z)};
        add(d.x, f1);
        add(d.y, f2);
        add(d.z, f3);
        add(d.w, f4);
    }
}


constexpr int kUsThreads = 256;

// Centre of mass of both restraint groups of window w in FP64, reduced by one
// block in a fixed order (us_force_cuda.cu:14-48, whose __syncthreads only
// orders a single block); writes the COMs and the CV of the window and returns
// (in `sf`, on every thread) the minimum-image COM axis r and (|r| - x0)/|r|.
__device__ void umbrella_com_block(const UmbrellaArgs &a, int w, double *s_red /* [6][kUsThreads] */,
                                   double *sf /* [4], shared */) {
    const WinDev W = a.win[w];
    double c[6] = {0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < W.n_bias; b += blockDim.x) {
        const int2 e = a.bias[W.bias_off + b];
        const float4 x = a.pos[e.x];
        const double m = a.mfrac[W.bias_off + b];
        const int o = 3 * e.y;
        c[o + 0] += m * x.x;
        c[o + 1] += m * x.y;
        c[o + 2] += m * x.z;
    }
    for (int k = 0; k < 6; ++k) s_red[k * kUsThreads + threadIdx.x] = c[k];
    for (int t = threadIdx.x + blockDim.x; t < kUsThreads; t += blockDim.x)
        for (int k = 0; k < 6; ++k) s_red[k * kUsThreads + t] = 0.0;
    __syncthreads();
    for (int stride = kUsThreads / 2; stride > 0; stride >>= 1) {
        for (int t = threadIdx.x; t < stride; t += blockDim.x)
            for (int k = 0; k < 6; ++k) s_red[k * kUsThreads + t] += s_red[k * kUsThreads + t + stride];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double L = W.box, hh = 0.5 * W.box;
        double r[3];
        for (int k = 0; k < 3; ++k) {
            double v = s_red[k * kUsThreads] - s_red[(3 + k) * kUsThreads];
            if (v > hh) v -= L;
            else if (v < -hh) v += L;
            r[k] = v;
        }
        const double d = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        for (int k = 0; k < 6; ++k) a.com[6 * (long long)w + k] = s_red[k * kUsThreads];
        a.cv[w] = d;
        sf[0] = r[0];
        sf[1] = r[1];
        sf[2] = r[2];
        sf[3] = (d - (double)W.us_x0) / d;
    }
    __syncthreads();
}

// Restraint force on bias entry b of window w: -+k (d - x0)/d m_i/M_g r
// (us_class.cpp:153-154 sign per group), in the accumulator's fixed point.
__device__ __forceinline__ void umbrella_entry_fix(const UmbrellaArgs &a, const WinDev &W, int b, const double *sf,
                                                   long long out[3]) {
    const int2 e = a.bias[W.bias_off + b];
    const double ku = e.y == 0 ? -(double)W.us_k : (double)W.us_k;
    const double pf = ku * sf[3] * (double)a.mfrac[W.bias_off + b];
    const double f[3] = {pf * sf[0], pf * sf[1], pf * sf[2]};
    const double m = fmax(fabs(f[0]), fmax(fabs(f[1]), fabs(f[2])));
    if (!(m <= (double)kFixLimit)) atomicOr(a.status, (m != m || isinf(m)) ? kStatusNonFinite : kStatusOverflow);
    for (int k = 0; k < 3; ++k) out[k] = __double2ll_rn(f[k] * 4294967296.0);
}


// Leapfrog of atom i (leapfrog_cuda.cu:33-68) from the accumulated force
// plus `extra` (fixed point), which it reads through L2 and clears.

__device__ __forceinline__ void leapfrog_atom(const LeapfrogArgs &a, int i, uint32_t step, const long long *extra) {
    const int w = a.atom_win[i];
    const WinDev W = a.win[w];
    unsigned long long *acc = a.facc + 3 * (long long)i;
    long long s[3] = {(long long)__ldcg(acc + 0), (long long)__ldcg(acc + 1), (long long)__ldcg(acc + 2)};
    if (extra)
        for (int k = 0; k < 3; ++k) s[k] += extra[k];
    const float fx = (float)((double)s[0] * kFixInv);
    const float fy = (float)((double)s[1] * kFixInv);
    const float fz = (float)((double)s[2] * kFixInv);
    acc[0] = 0ull;
    acc[1] = 0ull;
    acc[2] = 0ull;
    a.force_out[i] = make_float4(fx, fy, fz, 0.0f);
    float4 v = a.vel[i];
    float4 x = a.pos[i];
    const uint32_t il = (uint32_t)(i - W.atom_off);
    const uint32_t ctr3 = ((uint32_t)w << 8) | 1u;
    const u32x4 o = philox4x32_10(u32x4{il, 0u, step, ctr3}, a.seed_lo, a.seed_hi);
    const float m = v.w;
    if (u01(o.x) < W.pnu) {  // Andersen collision (:50-56)
        const u32x4 g = philox4x32_10(u32x4{il, 1u, step, ctr3}, a.seed_lo, a.seed_hi);
        const float ra = sqrtf(-2.0f * logf(u01_open0(g.x)));
        const float rb = sqrtf(-2.0f * logf(u01_open0(g.z)));
        float s1, c1, s3, c3;
        sincospif(2.0f * u01_open0(g.y), &s1, &c1);
        sincospif(2.0f * u01_open0(g.w), &s3, &c3);
        const float sd = sqrtf(W.kT / m);
        const float hk = W.dt / (2.0f * m);
        v.x = ra * c1 * sd + fx * hk;
        v.y = ra * s1 * sd + fy * hk;
        v.z = rb * c3 * sd + fz * hk;
    } else {
        const float k = W.dt / m;
        v.x += fx * k;
        v.y += fy * k;
        v.z += fz * k;
    }
    x.x += v.x * W.dt;
    x.y += v.y * W.dt;
    x.z += v.z * W.dt;
    // wrap (cuda_vector_routines.h wrap)
    const float L = W.box;
    x.x = x.x > L ? x.x - L : (x.x < 0.0f ? x.x + L : x.x);
    x.y = x.y > L ? x.y - L : (x.y < 0.0f ? x.y + L : x.y);
    x.z = x.z > L ? x.z - L : (x.z < 0.0f ? x.z + L : x.z);
    if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z)))
        atomicOr(a.status, kStatusNonFinite);
    a.vel[i] = v;
    a.pos[i] = x;
}

// Grid-wide barrier of a cooperative launch (every block resident): arrival
// count and generation word, both zero at rest.  The wait is bounded: after
// kBarrierWaitNs of global time the block gives up, flags kStatusTimeout and
// returns false, and the caller skips the work that needed the barrier.
constexpr unsigned long long kBarrierWaitNs = 500000000ull;
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ bool grid_barrier(unsigned int *bar, int *status) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *gen = bar + 1;
        const unsigned int g = *gen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (*gen == g) {
                if (global_ns() - t0 > kBarrierWaitNs) {
                    atomicOr(status, kStatusTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}


// The fused integrator's phases, shared with the single-kernel step.
// Restrained windows' COM axes into usf, one block per window in a fixed order.
__device__ __forceinline__ void restraint_coms(const IntegratorArgs &a) {
    __shared__ double s_red[6 * kUsThreads];
    __shared__ double s_f[4];
    for (int u = blockIdx.x; u < a.us.n_us_windows; u += gridDim.x) {
        const int w = a.us.us_windows[u];
        umbrella_com_block(a.us, w, s_red, s_f);
        if (threadIdx.x == 0) {
            a.usf[2 * w] = make_double2(s_f[0], s_f[1]);
            a.usf[2 * w + 1] = make_double2(s_f[2], s_f[3]);
        }
        __syncthreads();
    }
}
// Every enabled bonded term, spread over the grid's threads.
__device__ __forceinline__ void bonded_terms(const BondedArgs &b) {
    const long long n_terms = (b.do_bonds ? b.n_bonds : 0) + (b.do_angles ? b.n_angles : 0) + (b.do_dihs ? b.n_dihs : 0);
    const long long stride = (long long)gridDim.x * blockDim.x;
    const FixAdd add{b.facc, b.status};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n_terms; t += stride)
        bonded_term(b, t, add);
}
// After the grid barrier: every atom adds its restraint force from its
// window's COM axis (the umbrella kernel's fixed-point values) and is
// integrated; block 0 advances the step counter (every block read it before
// the barrier).
__device__ __forceinline__ void integrate_atoms(const IntegratorArgs &a, uint32_t step) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.lf.n_atoms; i += stride) {
        long long extra[3] = {0, 0, 0};
        for (int k = a.bias_start[i]; k < a.bias_start[i + 1]; ++k) {
            const int b = a.bias_by_atom[k];  // global bias entry
            const int w = a.lf.atom_win[i];
            const WinDev W = a.us.win[w];
            const double2 q0 = __ldcg(a.usf + 2 * w), q1 = __ldcg(a.usf + 2 * w + 1);
            const double sf[4] = {q0.x, q0.y, q1.x, q1.y};
            long long f[3];
            umbrella_entry_fix(a.us, W, b - W.bias_off, sf, f);
            for (int c = 0; c < 3; ++c) extra[c] += f[c];
        }
        leapfrog_atom(a.lf, (int)i, step, extra);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *a.lf.step_ptr = step + 1u;
        if (a.lf.ov_epoch) ++*a.lf.ov_epoch;
    }
}

}  // namespace
}  // namespace isspa
