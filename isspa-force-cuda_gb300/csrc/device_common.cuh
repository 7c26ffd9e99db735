// device_common.cuh -- device-side layouts and helpers shared by the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace isspa {

// IS-SPA constants, src/constants.h:6-13 of the reference (float literals).
constexpr float kEp = 2.3473f;
constexpr float kRho = 0.0075f;
constexpr float kP0 = 4.173705894203977f;
constexpr float kQ0 = 1.6899960102882601f;
constexpr float kO0 = 9.3658298730779350f;
constexpr float kPi = 3.1415926535f;

// Fixed-point force accumulation: 32 fractional bits in a signed 64-bit word.
// Integer addition is associative, so the summed force is bit-identical for
// any order of the atomics.
constexpr float kFixScale = 4294967296.0f;
constexpr double kFixInv = 1.0 / 4294967296.0;
constexpr float kFixLimit = 1.0e9f;  // |f| beyond this flags ISSPA_ERR_OVERFLOW

// Device status bits (sticky, read by the host after a step).
enum : int {
    kStatusOverflow = 1,
    kStatusNonFinite = 2,
    kStatusBounds = 4,
    kStatusTimeout = 8,  // a bounded device wait gave up
    kStatusListFull = 16,  // a neighbour-list row outgrew its capacity
};

// Programmatic dependent launch.  A kernel launched as a programmatic
// dependent of the kernel before it on the stream may be scheduled while that
// kernel still runs; pdl_wait() returns once every kernel it depends on has
// completed and its memory is visible (at once for an ordinary launch), so it
// comes before the kernel's first global access.  pdl_trigger() lets the next
// kernel's blocks be scheduled once every block of this one has passed it.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// One window (umbrella window or replica) of a batch.
struct WinDev {
    int atom_off, n_atoms;     // global atom range
    long long point_off;       // first MC point (global)
    float box, hbox;
    float kT, dt, pnu;
    int bias_off, n_bias;      // umbrella atoms (global list range)
    float us_k, us_x0;
    int us_on;
    int pad;
};

// Packed per-point results of the field pass, consumed by the force pass.
// With a_1 = p0<P1> w/n, a_2 = q0<P2> w/n, a_3 = o0<P3> w/n (the reference's
// dipole / quadrupole / octupole amplitudes over rho, isspa_force_cuda.cu:
// 279-287) the force of point p on atom i, per unit -q_i vtot_i, is
//   r ri^5 [3 (D.r) + w g (7.5 a2 + 17.5 a3 g) - 1.5 a2 - 7.5 a3 g]
//   - E^ ri^3 [g (3 a2 + 7.5 a3 g) - 1.5 a3 ri^2] - D ri^3,
// w = E^.r, g = w ri^2, with the dipole vector D = a1 E^ inside rmax of the
// atom's type and D = a1 E^ + p0 E0/(3n) outside: the constant-density
// dielectric term (:306-312) is a dipole field of moment p0 E0/(3n) and folds
// into the multipole's dipole term.
struct PointsDev {
    float4 *q0;   // x, y, z, w/n                 (position, density per unit vtot)
    float4 *q1;   // E^x, E^y, E^z, 1.5 a2
    float4 *q2;   // 7.5 a2, 17.5 a3, 3 a2, 7.5 a3
    float4 *q3;   // D (inside rmax), 1.5 a3
    float4 *q4;   // D (outside rmax), 1.5 a3
};

// Minimum image at most one box away (the reference's min_image): identical
// result to `r > h ? r - L : (r < -h ? r + L : r)`.
__device__ __forceinline__ float mimg(float r, float L, float h) {
    return fabsf(r) > h ? r - copysignf(L, r) : r;
}
// Distance that picks a density-table bin in the field pass: r^2 times the
// reciprocal square root the caller already holds (within a few ulp of the
// correctly rounded root, as the reference's fast-math sqrtf).  The density
// table is interpolated between bin and bin + 1 with the bin truncated
// (isspa_force_cuda.cu:157-167), which is continuous across bin edges, so a bin
// picked one rounding step off moves the result by rounding only.  The
// mean-force table rounds to the nearest bin and interpolates from there
// (:292-301), which jumps at half-bin edges: its distance stays the correctly
// rounded root, the bin the oracle picks (so does the adjoint's).
__device__ __forceinline__ float density_table_dist(float d2, float ri) { return __fmul_rn(d2, ri); }
// Squared distance with a fixed operation sequence (no contraction freedom).
__device__ __forceinline__ float dist2f(float x, float y, float z) {
    return __fmaf_rn(z, z, __fmaf_rn(y, y, __fmul_rn(x, x)));
}

__device__ __forceinline__ long long to_fix(float v) { return __float2ll_rn(v * kFixScale); }

__device__ __forceinline__ void fix_add3(unsigned long long *acc, float fx, float fy, float fz) {
    atomicAdd(acc + 0, (unsigned long long)to_fix(fx));
    atomicAdd(acc + 1, (unsigned long long)to_fix(fy));
    atomicAdd(acc + 2, (unsigned long long)to_fix(fz));
}

__device__ __forceinline__ void check_force(int *status, float fx, float fy, float fz) {
    float m = fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz)));
    if (!(m <= kFixLimit)) atomicOr(status, (m != m || isinf(m)) ? kStatusNonFinite : kStatusOverflow);
}

}  // namespace isspa
