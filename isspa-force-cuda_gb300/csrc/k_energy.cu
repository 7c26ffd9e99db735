// k_energy.cu -- potential and kinetic energies and the virial, FP64 reductions.
//
// The reference computes forces only; these kernels give the energies whose
// negative gradients are the reference's conservative forces, for energy
// conservation (NVE drift) checks:
//   pair:    LJ A/r^12 - B/r^6 and Coulomb q q/r over non-excluded pairs
//            (nonbond_force_cuda.cu:131-136), and the IS-SPA dielectric
//            correction (:141-147) integrated from infinity,
//              r > 2 rm:  U = -2 (1-1/ep) q q / (3 r)
//              r <= 2 rm: U = (1-1/ep) q q [(4 rm r^2 - r^3)/(24 rm^4) - 2/(3 rm)]
//            (continuous at 2 rm, rm the partner's rmax as in the force);
//   bonded:  k (r-r0)^2, k (theta-theta0)^2 with 2k stored
//            (bond_force_cuda.cu:36-50, angle_force_cuda.cu:19-52),
//            V (1 + cos(n phi - phase)) (dih_force_cuda.cu:86-135) and the
//            scaled 1-4 LJ and Coulomb (:60-82);
//   state:   m v^2/2 with v(t-dt/2) and with the thermostat-free kick
//            v(t+dt/2) = v(t-dt/2) + F(t) dt/m (leapfrog_cuda.cu:57-60), and
//            the umbrella k/2 (d - x0)^2 (us_force_cuda.cu:14-48).
// The virial is sum r . F over the same terms.  Pair energies are evaluated
// in FP32 with the force kernel's geometry and summed per stage of 128
// partners in FP32, then in FP64; bonded terms are FP64 throughout (as their
// forces); every cross-thread reduction is FP64 (warp shuffles, then one
// atomicAdd per warp or block and component).
#include <climits>
#include <cuda_runtime.h>

#include "kernels.h"

namespace isspa {
namespace {

constexpr int kEnThreads = 128;  // = the nonbond work items' atoms per item

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Adds v[k] into energy[w][slot[k]] for every lane with w >= 0.  When all
// contributing lanes of the warp share a window the warp reduces first and
// one lane adds.  Every lane of the warp must call this.
template <int NV>
__device__ __forceinline__ void window_add(double *energy, int w, const double (&v)[NV], const int (&slot)[NV]) {
    const unsigned act = __ballot_sync(0xffffffffu, w >= 0);
    if (!act) return;
    const int leader = __ffs(act) - 1;
    const int w0 = __shfl_sync(0xffffffffu, w, leader);
    if (__all_sync(0xffffffffu, w < 0 || w == w0)) {
        const bool lead = (int)(threadIdx.x & 31) == leader;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const double s = warp_sum(w >= 0 ? v[k] : 0.0);
            if (lead && s != 0.0) atomicAdd(energy + (long long)w0 * kECount + slot[k], s);
        }
    } else if (w >= 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            if (v[k] != 0.0) atomicAdd(energy + (long long)w * kECount + slot[k], v[k]);
    }
}

// Same work items and partner order as the nonbond force kernel; all atoms
// of an item belong to one window.  Ordered pairs, halved at the end.
__global__ void __launch_bounds__(kEnThreads) nonbond_energy_kernel(NonbondArgs a, double *energy) {
    __shared__ float4 s_x[kEnThreads];
    __shared__ float4 s_c[kEnThreads];  // rmax_j, (2 rmax_j)^2, 4 rmax_j, (1-1/ep)/(24 rmax_j^4)
    __shared__ float s_k[kEnThreads];   // 2 (1-1/ep) / (3 rmax_j)
    __shared__ int s_t[kEnThreads];
    __shared__ double s_red[4][kEnThreads / 32];
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

    int cur = a.excl_start[i];
    const int end = a.excl_start[i + 1];
    while (cur < end && a.excl[cur] < item.w) ++cur;
    int next_ex = cur < end ? a.excl[cur] : INT_MAX;

    double elj = 0.0, ecoul = 0.0, ecorr = 0.0, vir = 0.0;
    for (int j0 = 0; j0 < nj; j0 += kEnThreads) {
        const int jn = min(kEnThreads, nj - j0);
        float ulj = 0.f, uc = 0.f, ucr = 0.f, vr = 0.f;
        __syncthreads();
        if (t < jn) {
            const int j = item.w + j0 + t;
            s_x[t] = a.pos[j];
            const int2 ty = a.atype[j];
            const float rm = __ldg(a.rmax + ty.y);
            const float two = 2.0f * rm;
            const float r2 = rm * rm;
            s_c[t] = make_float4(rm, __fmul_rn(two, two), 4.0f * rm, epf / (24.0f * r2 * r2));
            s_k[t] = 2.0f * epf / (3.0f * rm);
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
            if (d2 >= a.cut2) continue;  // cutoff mode: the truncated potential
            const float ri = rsqrtf(d2);
            const float qq = xi.w * xj.w;
            if (terms & 4) {
                const float4 c = s_c[k];
                if (d2 > c.y) {
                    const float u = kfar * qq * ri;
                    ucr += u;
                    vr += u;  // r . F = -r dU/dr = U for a 1/r potential
                } else {
                    const float r = d2 * ri;
                    ucr += qq * (c.w * d2 * (c.z - r) - s_k[k]);
                    vr += -qq * c.w * d2 * (2.0f * c.z - 3.0f * r);
                }
            }
            if (!ex) {
                if (terms & 1) {
                    const float2 ab = __ldg(a.ljab + trow + s_t[k]);
                    const float ri2 = ri * ri;
                    const float r6 = ri2 * ri2 * ri2;
                    ulj += r6 * fmaf(ab.x, r6, -ab.y);
                    vr += r6 * fmaf(12.0f * ab.x, r6, -6.0f * ab.y);
                }
                if (terms & 2) {
                    uc += qq * ri;
                    vr += qq * ri;
                }
            }
        }
        elj += ulj;
        ecoul += uc;
        ecorr += ucr;
        vir += vr;
    }
    double v[4] = {active ? elj : 0.0, active ? ecoul : 0.0, active ? ecorr : 0.0, active ? vir : 0.0};
    const int lane = t & 31, wid = t >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = warp_sum(v[k]);
        if (lane == 0) s_red[k][wid] = v[k];
    }
    __syncthreads();
    if (t == 0) {
        const int slot[4] = {kELj, kECoul, kECorr, kEVirial};
        for (int k = 0; k < 4; ++k) {
            double s = 0.0;
            for (int q = 0; q < kEnThreads / 32; ++q) s += s_red[k][q];
            if (s != 0.0) atomicAdd(energy + (long long)item.x * kECount + slot[k], 0.5 * s);
        }
    }
}

__device__ __forceinline__ double3 rvec_d(const float4 *pos, int p, int q, float L, float h) {
    const float4 a = pos[p], b = pos[q];
    return make_double3(mimg(a.x - b.x, L, h), mimg(a.y - b.y, L, h), mimg(a.z - b.z, L, h));
}
__device__ __forceinline__ double dot3d(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__global__ void bonded_energy_kernel(BondedArgs a, double *energy) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nb = a.do_bonds ? a.n_bonds : 0;
    const long long na = a.do_angles ? a.n_angles : 0;
    const long long nd = a.do_dihs ? a.n_dihs : 0;
    double v[6] = {0, 0, 0, 0, 0, 0};  // bond, angle, dihedral, lj14, coul14, virial
    int w = -1;
    if (idx < nb) {
        const int4 b = a.bonds[idx];
        w = a.atom_win[b.x];
        const WinDev W = a.win[w];
        const double3 r = rvec_d(a.pos, b.x, b.y, W.box, W.hbox);
        const float2 p = a.bond_par[b.z];
        const double d = sqrt(dot3d(r, r)), dr = d - (double)p.y;
        v[0] = 0.5 * (double)p.x * dr * dr;
        v[5] = -(double)p.x * dr * d;  // r . F_x with F_x = 2k (r0/d - 1) r
    } else if ((idx -= nb) < na) {
        const int4 g = a.angles[idx];
        w = a.atom_win[g.x];
        const WinDev W = a.win[w];
        const double3 r1 = rvec_d(a.pos, g.x, g.y, W.box, W.hbox);
        const double3 r2 = rvec_d(a.pos, g.y, g.z, W.box, W.hbox);
        const double c11 = dot3d(r1, r1), c22 = dot3d(r2, r2), c12 = dot3d(r1, r2);
        const double b = -c12 / sqrt(c11 * c22);
        const double theta = b >= 1.0 ? 1.0e-16 : (b <= -1.0 ? (double)kPi : acos(b));
        const float2 p = a.angle_par[g.w];
        const double dt = theta - (double)p.y;
        v[1] = 0.5 * (double)p.x * dt * dt;
        const double f = (double)p.x * dt / sqrt(c11 * c22 - c12 * c12);
        const double a1 = c12 / c11, a2 = c12 / c22;
        const double3 Fx = make_double3(f * (a1 * r1.x - r2.x), f * (a1 * r1.y - r2.y), f * (a1 * r1.z - r2.z));
        const double3 Fz = make_double3(f * (r1.x - a2 * r2.x), f * (r1.y - a2 * r2.y), f * (r1.z - a2 * r2.z));
        v[5] = dot3d(r1, Fx) - dot3d(r2, Fz);  // x - y = r1, z - y = -r2
    } else if ((idx -= na) < nd) {
        const int4 d = a.dihs[idx];
        const int raw = a.dih_type[idx];
        const int ty = raw & 0x3FFFFFFF;
        w = a.atom_win[d.x];
        const WinDev W = a.win[w];
        const float L = W.box, h = W.hbox;
        if (raw & 0x40000000) {
            const float2 ab = __ldg(a.ljab + a.atype[d.x].x * a.n_lj_types + a.atype[d.w].x);
            const float2 sc = a.sc14[ty];
            const double3 r14 = rvec_d(a.pos, d.x, d.w, L, h);
            const double rm = dot3d(r14, r14);
            const double r6 = 1.0 / (rm * rm * rm);
            const double qq = (double)a.pos[d.x].w * (double)a.pos[d.w].w;
            v[3] = r6 * ((double)ab.x * r6 - (double)ab.y) / (double)sc.y;
            v[4] = qq / (sqrt(rm) * (double)sc.x);
            v[5] = 12.0 * r6 * r6 * (double)ab.x / (double)sc.y - 6.0 * r6 * (double)ab.y / (double)sc.y + v[4];
        }
        const double3 r12 = rvec_d(a.pos, d.x, d.y, L, h);
        const double3 r23 = rvec_d(a.pos, d.y, d.z, L, h);
        const double3 r34 = rvec_d(a.pos, d.z, d.w, L, h);
        const double c11 = dot3d(r12, r12), c22 = dot3d(r23, r23), c12 = dot3d(r12, r23);
        const double c33 = dot3d(r34, r34), c23 = dot3d(r23, r34), c13 = dot3d(r12, r34);
        const double t1 = c13 * c22 - c12 * c23;
        const double t2 = c11 * c23 - c12 * c13;
        const double t3 = c12 * c12 - c11 * c22;
        const double t4 = c22 * c33 - c23 * c23;
        const double t5 = c13 * c23 - c12 * c33;
        const double t6 = -t1;
        const double b = sqrt(-t3 * t4);
        const double cs = t6 / b;
        const float4 p = a.dih_par[ty];
        double fd = 0.0, phi = cs <= -1.0 ? (double)kPi : 0.0;
        if (cs > -1.0 && cs < 1.0) {
            phi = acos(cs);
            fd = (double)p.x * (double)p.y * sin((double)p.x * phi - (double)p.z) * c22 / (sin(phi) * b);
        }
        v[2] = (double)p.y * (1.0 + cos((double)p.x * phi - (double)p.z));
        const double g1 = fd / t3, g4 = -fd / t4;
        const double3 F1 = make_double3(g1 * (t1 * r12.x + t2 * r23.x + t3 * r34.x),
                                        g1 * (t1 * r12.y + t2 * r23.y + t3 * r34.y),
                                        g1 * (t1 * r12.z + t2 * r23.z + t3 * r34.z));
        const double3 F4 = make_double3(g4 * (t4 * r12.x + t5 * r23.x + t6 * r34.x),
                                        g4 * (t4 * r12.y + t5 * r23.y + t6 * r34.y),
                                        g4 * (t4 * r12.z + t5 * r23.z + t6 * r34.z));
        const double u = c12 / c22, vv = c23 / c22;
        const double3 F3 = make_double3(u * F1.x - (1.0 + vv) * F4.x, u * F1.y - (1.0 + vv) * F4.y,
                                        u * F1.z - (1.0 + vv) * F4.z);
        // x - y = r12, z - y = -r23, w - y = -(r23 + r34)
        const double3 r24 = make_double3(r23.x + r34.x, r23.y + r34.y, r23.z + r34.z);
        v[5] += dot3d(r12, F1) - dot3d(r23, F3) - dot3d(r24, F4);
    }
    const int slot[6] = {kEBond, kEAngle, kEDihedral, kELj14, kECoul14, kEVirial};
    window_add(energy, w, v, slot);
}

__global__ void state_energy_kernel(StateEnergyArgs a, double *energy) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    int w = -1;
    if (i < a.n_atoms) {
        w = a.atom_win[i];
        const WinDev W = a.win[w];
        const float4 vel = a.vel[i];
        const unsigned long long *acc = a.facc + 3 * (long long)i;
        // the integrator's own arithmetic for the kick (k_md.cu leapfrog_atom)
        const float fx = (float)((double)(long long)acc[0] * kFixInv);
        const float fy = (float)((double)(long long)acc[1] * kFixInv);
        const float fz = (float)((double)(long long)acc[2] * kFixInv);
        const float m = vel.w, k = W.dt / m;
        const float px = vel.x + fx * k, py = vel.y + fy * k, pz = vel.z + fz * k;
        const double hm = 0.5 * (double)m;
        v[0] = hm * ((double)vel.x * vel.x + (double)vel.y * vel.y + (double)vel.z * vel.z);
        v[1] = hm * ((double)px * px + (double)py * py + (double)pz * pz);
    }
    const int slot[2] = {kEKinBefore, kEKinAfter};
    window_add(energy, w, v, slot);
    if (blockIdx.x == 0)
        for (int k = threadIdx.x; k < a.n_us_windows; k += blockDim.x) {
            const int uw = a.us_windows[k];
            const WinDev W = a.win[uw];
            const double d = a.cv[uw], dx = d - (double)W.us_x0;
            atomicAdd(energy + (long long)uw * kECount + kEUmbrella, 0.5 * (double)W.us_k * dx * dx);
            atomicAdd(energy + (long long)uw * kECount + kEVirial, -(double)W.us_k * dx * d);
        }
}

}  // namespace

void launch_nonbond_energy(const NonbondArgs &a, double *energy, cudaStream_t s) {
    if (a.n_items > 0) nonbond_energy_kernel<<<a.n_items, kEnThreads, 0, s>>>(a, energy);
}

void launch_bonded_energy(const BondedArgs &a, double *energy, cudaStream_t s) {
    const long long n = (a.do_bonds ? a.n_bonds : 0) + (a.do_angles ? a.n_angles : 0) + (a.do_dihs ? a.n_dihs : 0);
    if (n > 0) bonded_energy_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a, energy);
}

void launch_state_energy(const StateEnergyArgs &a, double *energy, cudaStream_t s) {
    const int blocks = a.n_atoms > 0 ? (a.n_atoms + 127) / 128 : 1;
    state_energy_kernel<<<blocks, 128, 0, s>>>(a, energy);
}

}  // namespace isspa
