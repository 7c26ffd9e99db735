// k_md.cu -- pair, bonded, umbrella and integrator kernels for sm_103a.
//
//  nonbond:  all-pairs LJ + Coulomb + IS-SPA long-range dielectric correction
//            (reference src/nonbond_force_cuda.cu:31-174).  One thread per
//            receiving atom, partner atoms streamed through shared memory,
//            exclusions from a per-atom sorted list walked with a cursor (the
//            reference copies the whole list into shared memory per block and
//            fails once it exceeds 48 KB).
//  bonded:   bonds, angles, dihedrals with scaled 1-4 (bond_force_cuda.cu:
//            15-53, angle_force_cuda.cu:12-66, dih_force_cuda.cu:13-136) in one
//            launch over the concatenated term lists.
//  umbrella: one block per restrained window: FP64 centre-of-mass reduction,
//            then the harmonic COM-distance force (us_force_cuda.cu:14-48,
//            whose __syncthreads only orders a single block).
//  leapfrog: consumes and clears the fixed-point force accumulator, Andersen
//            collisions from Philox, leapfrog update and wrap
//            (leapfrog_cuda.cu:33-68).
#include <climits>
#include <cuda_runtime.h>

#include "kernels.h"
#include "philox.h"

namespace isspa {

namespace {

constexpr int kNbThreads = 128;

__global__ void __launch_bounds__(kNbThreads) nonbond_kernel(NonbondArgs a) {
    __shared__ float4 s_x[kNbThreads];
    __shared__ float4 s_c[kNbThreads];  // rmax_j, (2 rmax_j)^2, 8 rmax_j, (1-1/ep)/(24 rmax_j^4)
    __shared__ int s_t[kNbThreads];
    const int4 item = a.items[blockIdx.x];
    const int nj = a.items_nj[blockIdx.x];
    const WinDev W = a.win[item.x];
    const int t = threadIdx.x;
    const bool active = t < item.z;
    const int i = item.y + (active ? t : 0);
    const float4 xi = a.pos[i];
    const int trow = a.atype[i].x * a.n_lj_types;
    const float L = W.box, h = W.hbox;
    const int terms = a.terms;
    const float epf = 1.0f - 1.0f / kEp;
    const float kfar = -2.0f * epf / 3.0f;

    // exclusion cursor: first entry >= first partner of this item
    int cur = a.excl_start[i];
    const int end = a.excl_start[i + 1];
    while (cur < end && a.excl[cur] < item.w) ++cur;
    int next_ex = cur < end ? a.excl[cur] : INT_MAX;

    long long fxa = 0, fya = 0, fza = 0;  // per-stage partial sums in fixed point
    for (int j0 = 0; j0 < nj; j0 += kNbThreads) {
        const int jn = min(kNbThreads, nj - j0);
        float ax = 0.f, ay = 0.f, az = 0.f;
        __syncthreads();
        if (t < jn) {
            const int j = item.w + j0 + t;
            s_x[t] = a.pos[j];
            const int2 ty = a.atype[j];
            const float rm = __ldg(a.rmax + ty.y);
            const float two = 2.0f * rm;
            const float r2 = rm * rm;
            s_c[t] = make_float4(rm, __fmul_rn(two, two), 8.0f * rm, epf / (24.0f * r2 * r2));
            s_t[t] = ty.x;
        }
        __syncthreads();
        for (int k = 0; k < jn; ++k) {
            const int j = item.w + j0 + k;
            const bool ex = j == next_ex;
            if (ex) {
                ++cur;
                next_ex = cur < end ? a.excl[cur] : INT_MAX;
            }
            if (j == i) continue;
            const float4 xj = s_x[k];
            const float rx = mimg(xi.x - xj.x, L, h);
            const float ry = mimg(xi.y - xj.y, L, h);
            const float rz = mimg(xi.z - xj.z, L, h);
            const float d2 = dist2f(rx, ry, rz);
            const float ri = rsqrtf(d2);
            const float ri2 = ri * ri;
            const float qq = xi.w * xj.w;
            float fs = 0.0f;
            if (terms & 4) {  // IS-SPA long-range dielectric correction (:141-147)
                const float4 c = s_c[k];
                fs = d2 > c.y ? kfar * qq * ri2 * ri : -qq * c.w * (c.z - 3.0f * d2 * ri);
            }
            if (!ex) {
                if (terms & 1) {  // LJ (:131-132)
                    const float2 ab = __ldg(a.ljab + trow + s_t[k]);
                    const float r6 = ri2 * ri2 * ri2;
                    fs += r6 * fmaf(12.0f * ab.x, r6, -6.0f * ab.y) * ri2;
                }
                if (terms & 2) fs += qq * ri2 * ri;  // Coulomb (:136)
            }
            ax = fmaf(fs, rx, ax);
            ay = fmaf(fs, ry, ay);
            az = fmaf(fs, rz, az);
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

// Image vector in float (the reference's minimum-image decision), then the
// bonded arithmetic in FP64: these terms are O(N) work, and acos / 1/sin(phi)
// / 1/|r12 x r23| make the FP32 formulas ill-conditioned for near-planar or
// near-linear geometries.
__device__ __forceinline__ double3 rvec(const float4 *pos, int p, int q, float L, float h) {
    const float4 a = pos[p], b = pos[q];
    return make_double3(mimg(a.x - b.x, L, h), mimg(a.y - b.y, L, h), mimg(a.z - b.z, L, h));
}

__device__ __forceinline__ void add_force(unsigned long long *facc, int *status, int atom, double fx,
                                          double fy, double fz) {
    const double m = fmax(fabs(fx), fmax(fabs(fy), fabs(fz)));
    if (!(m <= (double)kFixLimit)) atomicOr(status, (m != m || isinf(m)) ? kStatusNonFinite : kStatusOverflow);
    unsigned long long *acc = facc + 3 * (long long)atom;
    atomicAdd(acc + 0, (unsigned long long)__double2ll_rn(fx * 4294967296.0));
    atomicAdd(acc + 1, (unsigned long long)__double2ll_rn(fy * 4294967296.0));
    atomicAdd(acc + 2, (unsigned long long)__double2ll_rn(fz * 4294967296.0));
}

__device__ __forceinline__ double dot3(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__global__ void bonded_kernel(BondedArgs a) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nb = a.do_bonds ? a.n_bonds : 0;
    const long long na = a.do_angles ? a.n_angles : 0;
    const long long nd = a.do_dihs ? a.n_dihs : 0;
    if (idx < nb) {  // bond_force_cuda.cu:36-50: f = 2k (r0/|r| - 1) r on atom x
        const int4 b = a.bonds[idx];
        const WinDev W = a.win[a.atom_win[b.x]];
        const double3 r = rvec(a.pos, b.x, b.y, W.box, W.hbox);
        const float2 p = a.bond_par[b.z];
        const double f = (double)p.x * ((double)p.y / sqrt(dot3(r, r)) - 1.0);
        add_force(a.facc, a.status, b.x, f * r.x, f * r.y, f * r.z);
        add_force(a.facc, a.status, b.y, -f * r.x, -f * r.y, -f * r.z);
        return;
    }
    idx -= nb;
    if (idx < na) {  // angle_force_cuda.cu:19-52
        const int4 g = a.angles[idx];
        const WinDev W = a.win[a.atom_win[g.x]];
        const double3 r1 = rvec(a.pos, g.x, g.y, W.box, W.hbox);
        const double3 r2 = rvec(a.pos, g.y, g.z, W.box, W.hbox);
        const double c11 = dot3(r1, r1), c22 = dot3(r2, r2), c12 = dot3(r1, r2);
        const double b = -c12 / sqrt(c11 * c22);
        const double theta = b >= 1.0 ? 1.0e-16 : (b <= -1.0 ? (double)kPi : acos(b));
        const float2 p = a.angle_par[g.w];
        const double f = (double)p.x * (theta - (double)p.y) / sqrt(c11 * c22 - c12 * c12);
        const double a1 = c12 / c11, a2 = c12 / c22;
        add_force(a.facc, a.status, g.x, f * (a1 * r1.x - r2.x), f * (a1 * r1.y - r2.y), f * (a1 * r1.z - r2.z));
        add_force(a.facc, a.status, g.y, f * ((1.0 + a2) * r2.x - (1.0 + a1) * r1.x),
                  f * ((1.0 + a2) * r2.y - (1.0 + a1) * r1.y), f * ((1.0 + a2) * r2.z - (1.0 + a1) * r1.z));
        add_force(a.facc, a.status, g.z, f * (r1.x - a2 * r2.x), f * (r1.y - a2 * r2.y), f * (r1.z - a2 * r2.z));
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
            const double3 r14 = rvec(a.pos, d.x, d.w, L, h);
            const double rm = dot3(r14, r14);
            const double r6 = 1.0 / (rm * rm * rm);
            const double fe = (double)a.pos[d.x].w * (double)a.pos[d.w].w / (rm * sqrt(rm) * (double)sc.x);
            const double fv = r6 * (12.0 * (double)ab.x * r6 - 6.0 * (double)ab.y) / ((double)sc.y * rm);
            const double f = fe + fv;
            add_force(a.facc, a.status, d.x, f * r14.x, f * r14.y, f * r14.z);
            add_force(a.facc, a.status, d.w, -f * r14.x, -f * r14.y, -f * r14.z);
        }
        const double3 r12 = rvec(a.pos, d.x, d.y, L, h);
        const double3 r23 = rvec(a.pos, d.y, d.z, L, h);
        const double3 r34 = rvec(a.pos, d.z, d.w, L, h);
        const double c11 = dot3(r12, r12), c22 = dot3(r23, r23), c12 = dot3(r12, r23);
        const double c33 = dot3(r34, r34), c23 = dot3(r23, r34), c13 = dot3(r12, r34);
        const double t1 = c13 * c22 - c12 * c23;
        const double t2 = c11 * c23 - c12 * c13;
        const double t3 = c12 * c12 - c11 * c22;
        const double t4 = c22 * c33 - c23 * c23;
        const double t5 = c13 * c23 - c12 * c33;
        const double t6 = -t1;
        const double b = sqrt(-t3 * t4);
        const double cs = t6 / b;
        double fd = 0.0;
        if (cs > -1.0 && cs < 1.0) {
            const double phi = acos(cs);
            const float4 p = a.dih_par[ty];
            fd = (double)p.x * (double)p.y * sin((double)p.x * phi - (double)p.z) * c22 / (sin(phi) * b);
        }
        const double g1 = fd / t3, g4 = -fd / t4;
        const double f1x = g1 * (t1 * r12.x + t2 * r23.x + t3 * r34.x);
        const double f1y = g1 * (t1 * r12.y + t2 * r23.y + t3 * r34.y);
        const double f1z = g1 * (t1 * r12.z + t2 * r23.z + t3 * r34.z);
        const double f4x = g4 * (t4 * r12.x + t5 * r23.x + t6 * r34.x);
        const double f4y = g4 * (t4 * r12.y + t5 * r23.y + t6 * r34.y);
        const double f4z = g4 * (t4 * r12.z + t5 * r23.z + t6 * r34.z);
        const double u = c12 / c22, v = c23 / c22;
        add_force(a.facc, a.status, d.x, f1x, f1y, f1z);
        add_force(a.facc, a.status, d.y, -(1.0 + u) * f1x + v * f4x, -(1.0 + u) * f1y + v * f4y,
                  -(1.0 + u) * f1z + v * f4z);
        add_force(a.facc, a.status, d.z, u * f1x - (1.0 + v) * f4x, u * f1y - (1.0 + v) * f4y,
                  u * f1z - (1.0 + v) * f4z);
        add_force(a.facc, a.status, d.w, f4x, f4y, f4z);
    }
}

constexpr int kUsThreads = 256;

__global__ void __launch_bounds__(kUsThreads) umbrella_kernel(UmbrellaArgs a) {
    __shared__ double s_red[6][kUsThreads];
    __shared__ double s_f[4];
    const int w = a.us_windows[blockIdx.x];
    const WinDev W = a.win[w];
    double c[6] = {0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < W.n_bias; b += kUsThreads) {
        const int2 e = a.bias[W.bias_off + b];
        const float4 x = a.pos[e.x];
        const double m = a.mfrac[W.bias_off + b];
        const int o = 3 * e.y;
        c[o + 0] += m * x.x;
        c[o + 1] += m * x.y;
        c[o + 2] += m * x.z;
    }
    for (int k = 0; k < 6; ++k) s_red[k][threadIdx.x] = c[k];
    __syncthreads();
    for (int stride = kUsThreads / 2; stride > 0; stride >>= 1) {
        if (threadIdx.x < stride)
            for (int k = 0; k < 6; ++k) s_red[k][threadIdx.x] += s_red[k][threadIdx.x + stride];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double L = W.box, hh = 0.5 * W.box;
        double r[3];
        for (int k = 0; k < 3; ++k) {
            double v = s_red[k][0] - s_red[3 + k][0];
            if (v > hh) v -= L;
            else if (v < -hh) v += L;
            r[k] = v;
        }
        const double d = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        for (int k = 0; k < 6; ++k) a.com[6 * (long long)w + k] = s_red[k][0];
        a.cv[w] = d;
        s_f[0] = r[0];
        s_f[1] = r[1];
        s_f[2] = r[2];
        s_f[3] = (d - (double)W.us_x0) / d;
    }
    __syncthreads();
    for (int b = threadIdx.x; b < W.n_bias; b += kUsThreads) {
        const int2 e = a.bias[W.bias_off + b];
        const double ku = e.y == 0 ? -(double)W.us_k : (double)W.us_k;  // us_class.cpp:153-154
        const double pf = ku * s_f[3] * (double)a.mfrac[W.bias_off + b];
        add_force(a.facc, a.status, e.x, pf * s_f[0], pf * s_f[1], pf * s_f[2]);
    }
}

__device__ __forceinline__ void leapfrog_atom(const LeapfrogArgs &a, int i, uint32_t step);

// Every block reads the step counter first; the last block to finish
// advances it (no block waits on another).
__global__ void leapfrog_kernel(LeapfrogArgs a) {
    const uint32_t step = *a.step_ptr;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n_atoms) leapfrog_atom(a, i, step);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int prev = atomicAdd(a.done_ptr, 1u);
        if (prev == gridDim.x - 1) {
            *a.step_ptr = step + 1u;
            *a.done_ptr = 0u;
            __threadfence();
        }
    }
}

__device__ __forceinline__ void leapfrog_atom(const LeapfrogArgs &a, int i, uint32_t step) {
    const int w = a.atom_win[i];
    const WinDev W = a.win[w];
    unsigned long long *acc = a.facc + 3 * (long long)i;
    const float fx = (float)((double)(long long)acc[0] * kFixInv);
    const float fy = (float)((double)(long long)acc[1] * kFixInv);
    const float fz = (float)((double)(long long)acc[2] * kFixInv);
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

// Neighbour list of one window: one warp per atom, partners scanned in
// ascending order and appended with a warp ballot, so every row comes out
// sorted and identical run to run (the reference appends in atomic order,
// neighborlist_cuda.cu:85-96).
__global__ void neighbor_list_kernel(ListArgs a) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= a.n_atoms) return;
    const int i = a.atom_off + warp;
    const float4 xi = a.pos[i];
    const int ex0 = a.excl_start[i], ex1 = a.excl_start[i + 1];
    int count = 0;
    for (int j0 = 0; j0 < a.n_atoms; j0 += 32) {
        const int jl = j0 + lane;
        bool hit = false;
        if (jl < a.n_atoms && jl != warp) {
            const int j = a.atom_off + jl;
            const float4 xj = a.pos[j];
            const float rx = mimg(xi.x - xj.x, a.box, a.hbox);
            const float ry = mimg(xi.y - xj.y, a.box, a.hbox);
            const float rz = mimg(xi.z - xj.z, a.box, a.hbox);
            hit = dist2f(rx, ry, rz) < a.rnn2;
            if (hit)
                for (int e = ex0; e < ex1; ++e)
                    if (a.excl[e] == j) {
                        hit = false;
                        break;
                    }
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int slot = count + __popc(m & ((1u << lane) - 1u));
            if (slot < a.max_per_atom) a.rows[(long long)warp * a.max_per_atom + slot] = jl;
        }
        count += __popc(m);
    }
    if (lane == 0) a.counts[warp] = count;
}

__global__ void cell_index_kernel(const float4 *pos, int off, int n, float rc, int3 nc, int *cell) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = pos[off + i];
    // cell_list_cuda.cu:27-29
    cell[i] = (int)(x.x / rc) * nc.y * nc.z + (int)(x.y / rc) * nc.z + (int)(x.z / rc);
}

__global__ void fma_peak_kernel(float *out, int iters, float seed) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.999999f, c = 1.0e-7f;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

}  // namespace

int nonbond_block_threads() { return kNbThreads; }

void launch_nonbond(const NonbondArgs &a, cudaStream_t s) {
    if (a.n_items > 0) nonbond_kernel<<<a.n_items, kNbThreads, 0, s>>>(a);
}

void launch_bonded(const BondedArgs &a, cudaStream_t s) {
    long long n = (a.do_bonds ? a.n_bonds : 0) + (a.do_angles ? a.n_angles : 0) + (a.do_dihs ? a.n_dihs : 0);
    if (n <= 0) return;
    const int tpb = 128;
    bonded_kernel<<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, s>>>(a);
}

void launch_umbrella(const UmbrellaArgs &a, cudaStream_t s) {
    if (a.n_us_windows > 0) umbrella_kernel<<<a.n_us_windows, kUsThreads, 0, s>>>(a);
}

void launch_leapfrog(const LeapfrogArgs &a, cudaStream_t s) {
    if (a.n_atoms > 0) leapfrog_kernel<<<(a.n_atoms + 127) / 128, 128, 0, s>>>(a);
}

void launch_neighbor_list(const ListArgs &a, cudaStream_t s) {
    if (a.n_atoms <= 0) return;
    const long long threads = (long long)a.n_atoms * 32;
    neighbor_list_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(a);
}

void launch_cell_index(const float4 *pos, int off, int n, float rc, int3 nc, int *cell, cudaStream_t s) {
    if (n > 0) cell_index_kernel<<<(n + 127) / 128, 128, 0, s>>>(pos, off, n, rc, nc, cell);
}

__global__ void copy3_kernel(Copy3Args a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (a.src[k]) a.dst[k][i] = a.src[k][i];
}

void launch_copy3(const Copy3Args &a, cudaStream_t s) {
    if (a.n > 0) copy3_kernel<<<(a.n + 255) / 256, 256, 0, s>>>(a);
}

double measure_fp32_peak_tflops() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return -1.0;
    const int threads = 256, blocks = sms * 8, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_peak_kernel<<<blocks, threads>>>(out, 64, 1.0f);  // warm-up
    cudaEventRecord(e0);
    fma_peak_kernel<<<blocks, threads>>>(out, iters, 1.0f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
    const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
    return flops / (ms * 1e-3) / 1e12;
}

}  // namespace isspa
