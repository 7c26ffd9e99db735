// k_adjoint.cu -- reverse-mode gradient of the mean COM-axis force.
//
// For one frame, J = sum_i c_i . F_i with c_i = +n/2 on restraint group 0 and
// -n/2 on group 1 (n: unit COM separation).  Writing the IS-SPA force of point
// p on atom i as F_ip = s_p G_ip + H_ip (s_p = w_p/n_p; G the multipole and
// tabulated-LJ parts per unit density, H the constant-density dielectric part,
// reference src/isspa_force_cuda.cu:274-312):
//   lambda_p   = dJ/ds_p = sum_i c_i . G_ip                       (points kernel)
//   dJ/dT_f[k] = sum c_i . (-vtot_i s_p r/d) x lerp weight of entry k (points kernel)
//   dJ/dT_g[k] = sum_p lambda_p/n_p dw_p/dT_g[k], w_p = prod_j g_j  (density kernel)
//   dJ/dA, dJ/dB of the nonbond LJ (nonbond_force_cuda.cu:131-132) and of the
//   scaled 1-4 LJ (dih_force_cuda.cu:70-74), which are linear in A and B.
// MC points are the field pass's (regenerated from the Philox counters of the
// frame's step); gradients accumulate in FP64 per window.
#include <cuda_runtime.h>

#include "kernels.h"

namespace isspa {
namespace {

__device__ __forceinline__ void langevin_d(float x, double &p1, double &p2, double &p3) {
    // backward continued fraction of i_l/i_(l-1) (all terms positive)
    if (x < 5.0f) {
        double r = 0.0, r2 = 0.0, r3 = 0.0;
        for (int l = 24; l >= 1; --l) {
            r = (double)x / ((double)(2 * l + 1) + (double)x * r);
            if (l == 3) r3 = r;
            if (l == 2) r2 = r;
        }
        p1 = r;
        p2 = r * r2;
        p3 = r * r2 * r3;
    } else {
        const double X = x, c = 1.0 / tanh(X), ix = 1.0 / X;
        p1 = c - ix;
        p2 = 1.0 + 3.0 * ix * ix - 3.0 * c * ix;
        p3 = (1.0 + 15.0 * ix * ix) * c - 6.0 * ix - 15.0 * ix * ix * ix;
    }
}

__global__ void adjoint_points_kernel(AdjointArgs a) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n_points) return;
    const int w = a.point_win[p];
    const WinDev W = a.win[w];
    if (!W.us_on) return;
    const float4 raw = a.raw_e[p], raw0 = a.raw_e0[p];
    const float4 P = a.q0[p];
    const int n = (int)raw0.w;
    const double inv_n = 1.0 / (double)n, sp = (double)raw.w * inv_n;
    const double mag = sqrt((double)raw.x * raw.x + (double)raw.y * raw.y + (double)raw.z * raw.z);
    double p1, p2, p3;
    langevin_d((float)mag, p1, p2, p3);
    const double eh[3] = {mag > 0 ? raw.x / mag : 0.0, mag > 0 ? raw.y / mag : 0.0, mag > 0 ? raw.z / mag : 0.0};
    const float L = W.box, h = W.hbox;
    double lam = 0.0;
    for (int k = a.adj_off[w]; k < a.adj_off[w + 1]; ++k) {
        const int i = a.adj_atoms[k];
        const double c0 = a.cvec[3 * i], c1 = a.cvec[3 * i + 1], c2 = a.cvec[3 * i + 2];
        const float4 xi = a.pos[i];
        const int it = a.atype[i].y;
        const float rm = __ldg(a.rmax + it);
        const double vt = __ldg(a.vtot + it), qi = xi.w;
        const float rx = mimg(P.x - xi.x, L, h), ry = mimg(P.y - xi.y, L, h), rz = mimg(P.z - xi.z, L, h);
        const float d2 = dist2f(rx, ry, rz);
        const double r[3] = {rx, ry, rz};
        const double dd2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2], dd = sqrt(dd2);
        const double Rz = (eh[0] * r[0] + eh[1] * r[1] + eh[2] * r[2]) / dd;
        const double dp1 = 3.0 * Rz, dp2 = 7.5 * Rz * Rz - 1.5, dp3 = (17.5 * Rz * Rz - 7.5) * Rz;
        const double t1 = (double)kP0 * p1 / (dd2 * dd), t2 = (double)kQ0 * p2 / (dd2 * dd2),
                     t3 = (double)kO0 * p3 / (dd2 * dd2 * dd);
        double G = 0.0;
        const double cc[3] = {c0, c1, c2};
        for (int d = 0; d < 3; ++d) {
            const double mu = t1 * (r[d] * dp1 / dd - eh[d]) + t2 * (r[d] * dp2 / dd - dp1 * eh[d]) +
                              t3 * (r[d] * dp3 / dd - dp2 * eh[d]);
            G += cc[d] * (-qi * vt * mu);
        }
        if (d2 <= __fmul_rn(rm, rm)) {
            const float dist = __fsqrt_rn(d2);
            const int bin = (int)__fmaf_rn(__fsub_rn(dist, a.f_r0), a.f_inv, 0.5f);
            if (bin >= 0 && bin < a.n_f) {
                const double fr = (dd - ((double)a.f_r0 + bin * (double)a.f_dr)) / a.f_dr;
                const long long fi = (long long)it * a.n_f + bin;
                const float2 tv = __ldg(a.ftab + fi);
                const double tab = tv.x * (1.0 - fr) + tv.y * fr;
                const double cr = -vt * (c0 * r[0] + c1 * r[1] + c2 * r[2]) / dd;
                G += cr * tab;
                double *df = a.dJ_df + (long long)w * a.n_ftab;
                atomicAdd(df + fi, cr * sp * (1.0 - fr));
                if (fi + 1 < a.n_ftab) atomicAdd(df + fi + 1, cr * sp * fr);
            }
        }
        lam += G;
    }
    a.lam[p] = lam;
}

__global__ void adjoint_density_kernel(AdjointArgs a) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n_points) return;
    const int w = a.point_win[p];
    const WinDev W = a.win[w];
    if (!W.us_on) return;
    const double lam = a.lam[p];
    if (lam == 0.0) return;
    const float4 P = a.q0[p];
    const int n = (int)a.raw_e0[p].w;
    const double dJdw = lam / (double)n;
    const int owner = W.atom_off + (int)((p - W.point_off) / a.n_mc);
    const float rm = __ldg(a.rmax + a.atype[owner].y);
    const float rm2 = __fmul_rn(rm, rm);
    const float L = W.box, h = W.hbox;
    int zeros = 0, forced = 0;
    double prod = 1.0;
    double *dg = a.dJ_dg + (long long)w * a.n_gtab;
    for (int pass = 0; pass < 2; ++pass) {
        for (int j = W.atom_off; j < W.atom_off + W.n_atoms; ++j) {
            const float4 xj = a.pos[j];
            const float rx = mimg(P.x - xj.x, L, h), ry = mimg(P.y - xj.y, L, h), rz = mimg(P.z - xj.z, L, h);
            const float d2 = dist2f(rx, ry, rz);
            if (!(d2 <= rm2)) continue;
            const float dist = __fsqrt_rn(d2);
            const int bin = (int)__fmul_rn(__fsub_rn(dist, a.g_r0), a.g_inv);
            if (bin < 0) {
                forced = 1;
                continue;
            }
            if (bin >= a.n_g - 1) continue;
            const double dd = sqrt((double)rx * rx + (double)ry * ry + (double)rz * rz);
            const double fr = (dd - ((double)a.g_r0 + bin * (double)a.g_dr)) / a.g_dr;
            const long long gi = (long long)a.atype[j].y * a.n_g + bin;
            const double g0 = a.g_table[gi], g1 = gi + 1 < a.n_gtab ? a.g_table[gi + 1] : 0.0;
            const double g = g0 * (1.0 - fr) + g1 * fr;
            if (pass == 0) {
                if (g == 0.0) ++zeros;
                else prod *= g;
            } else {
                double others;
                if (forced || zeros >= 2) others = 0.0;
                else if (zeros == 1) others = g == 0.0 ? prod : 0.0;
                else others = prod / g;
                const double d = dJdw * others;
                if (d != 0.0) {
                    atomicAdd(dg + gi, d * (1.0 - fr));
                    if (gi + 1 < a.n_gtab) atomicAdd(dg + gi + 1, d * fr);
                }
            }
        }
    }
}

// Nonbond LJ coefficient adjoint for every weighted atom i (thread) against
// all atoms of its window; exclusions as the nonbond kernel.
__global__ void adjoint_pairs_kernel(AdjointArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n_adj) return;
    const int i = a.adj_atoms[k];
    const int w = a.atom_win[i];
    const WinDev W = a.win[w];
    const double c0 = a.cvec[3 * i], c1 = a.cvec[3 * i + 1], c2 = a.cvec[3 * i + 2];
    const float4 xi = a.pos[i];
    const int ti = a.atype[i].x;
    const float L = W.box, h = W.hbox;
    int cur = a.excl_start[i];
    const int end = a.excl_start[i + 1];
    double *dA = a.dJ_dA + (long long)w * a.n_ljtab, *dB = a.dJ_dB + (long long)w * a.n_ljtab;
    for (int j = W.atom_off; j < W.atom_off + W.n_atoms; ++j) {
        bool ex = false;
        while (cur < end && a.excl[cur] < j) ++cur;
        if (cur < end && a.excl[cur] == j) ex = true;
        if (j == i || ex) continue;
        const float4 xj = a.pos[j];
        const double rx = mimg(xi.x - xj.x, L, h), ry = mimg(xi.y - xj.y, L, h), rz = mimg(xi.z - xj.z, L, h);
        const double d2 = rx * rx + ry * ry + rz * rz;
        const double r6 = 1.0 / (d2 * d2 * d2);
        const double cr = c0 * rx + c1 * ry + c2 * rz;
        const int kk = a.nbp[ti * a.n_lj_types + a.atype[j].x];
        atomicAdd(dA + kk, cr * 12.0 * r6 * r6 / d2);
        atomicAdd(dB + kk, cr * -6.0 * r6 / d2);
    }
}

// Scaled 1-4 LJ coefficient adjoint (force +f r14 on atom x, -f r14 on atom w).
__global__ void adjoint_14_kernel(AdjointArgs a) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= a.n_dihs) return;
    const int raw = a.dih_type[d];
    if (!(raw & 0x40000000)) return;
    const int4 at = a.dihs[d];
    const double dc0 = a.cvec[3 * at.x] - a.cvec[3 * at.w], dc1 = a.cvec[3 * at.x + 1] - a.cvec[3 * at.w + 1],
                 dc2 = a.cvec[3 * at.x + 2] - a.cvec[3 * at.w + 2];
    if (dc0 == 0.0 && dc1 == 0.0 && dc2 == 0.0) return;
    const int w = a.atom_win[at.x];
    const WinDev W = a.win[w];
    const float4 px = a.pos[at.x], pw = a.pos[at.w];
    const double rx = mimg(px.x - pw.x, W.box, W.hbox), ry = mimg(px.y - pw.y, W.box, W.hbox),
                 rz = mimg(px.z - pw.z, W.box, W.hbox);
    const double rm = rx * rx + ry * ry + rz * rz;
    const double r6 = 1.0 / (rm * rm * rm);
    const double scnb = a.sc14[raw & 0x3FFFFFFF].y;
    const double cr = dc0 * rx + dc1 * ry + dc2 * rz;
    const int kk = a.nbp[a.atype[at.x].x * a.n_lj_types + a.atype[at.w].x];
    atomicAdd(a.dJ_dA + (long long)w * a.n_ljtab + kk, cr * 12.0 * r6 * r6 / (scnb * rm));
    atomicAdd(a.dJ_dB + (long long)w * a.n_ljtab + kk, cr * -6.0 * r6 / (scnb * rm));
}

}  // namespace

void launch_adjoint(const AdjointArgs &a, cudaStream_t s) {
    if (a.n_points > 0) {
        const unsigned blocks = (unsigned)((a.n_points + 127) / 128);
        adjoint_points_kernel<<<blocks, 128, 0, s>>>(a);
        adjoint_density_kernel<<<blocks, 128, 0, s>>>(a);
    }
    if (a.n_adj > 0) adjoint_pairs_kernel<<<(a.n_adj + 63) / 64, 64, 0, s>>>(a);
    if (a.n_dihs > 0) adjoint_14_kernel<<<(a.n_dihs + 127) / 128, 128, 0, s>>>(a);
}

}  // namespace isspa
