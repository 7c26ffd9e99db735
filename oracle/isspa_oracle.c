/*
 * isspa_oracle.c -- CPU oracle (test infrastructure only; see isspa_oracle.h).
 *
 * Plain-C restatement of the reference kernels.  Each function cites the
 * reference file:line it follows.  Built with -ffp-contract=off so that the
 * float geometry below is evaluated exactly as written (explicit fmaf where the
 * GPU kernels fuse), on x86-64 and aarch64 alike.
 */
#include "isspa_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* IS-SPA constants, src/constants.h:6-13 (float literals there). */
#define ORC_EP 2.3473f
#define ORC_RHO 0.0075f
#define ORC_P0 4.173705894203977f
#define ORC_Q0 1.6899960102882601f
#define ORC_O0 9.3658298730779350f
#define ORC_PI 3.1415926535f

static double orc_e0(void) {
    /* e0 = 3/(4*PI*rho*p0)*(1-1/ep), evaluated in float as the macro is. */
    float e0 = 3.0f / (4.0f * ORC_PI * ORC_RHO * ORC_P0) * (1.0f - 1.0f / ORC_EP);
    return (double)e0;
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---------------------------------------------------------------------------
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11).  Pinned by the Random123 known-answer vectors in tests.
 * ------------------------------------------------------------------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline float u24(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-08f; }
static inline double u24open(uint32_t x) { return ((double)(x >> 8) + 1.0) * 5.9604644775390625e-08; }

/* Minimum image, at most one box away (cuda_vector_routines.h:28-47 of the
 * reference, i.e. src/cuda_vector_routines.h min_image). */
static inline float mimg(float r, float L, float h) {
    if (r > h) return r - L;
    if (r < -h) return r + L;
    return r;
}
static inline float dist2f(float x, float y, float z) { return fmaf(z, z, fmaf(y, y, x * x)); }

/* ---------------------------------------------------------------------------
 * K1: MC points, src/isspa_force_cuda.cu:73-107.  Rejection-sampled uniform
 * ball r^2 < 0.99 (:92-97), scaled by rmax of the owner's type and translated
 * to the owner (:99-100).  The curand XORWOW stream is replaced by Philox keyed
 * by (seed, step, window, point, attempt).
 * ------------------------------------------------------------------------- */
void orc_mc_points(const orc_isspa_sys *s, int n_mc, uint64_t seed, uint32_t step,
                   uint32_t window, float *pts) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const long P = (long)s->n_atoms * n_mc;
#pragma omp parallel for schedule(static)
    for (long p = 0; p < P; ++p) {
        int a = (int)(p / n_mc);
        float rm = s->rmax[s->isspa_type[a]];
        float mx = 0.f, my = 0.f, mz = 0.f;
        int ok = 0;
        for (uint32_t att = 0; att < 64u && !ok; ++att) {
            uint32_t ctr[4] = {(uint32_t)p, att, step, (window << 8) | 0u}, o[4];
            orc_philox4x32_10(ctr, key, o);
            mx = fmaf(2.0f, u24(o[0]), -1.0f);
            my = fmaf(2.0f, u24(o[1]), -1.0f);
            mz = fmaf(2.0f, u24(o[2]), -1.0f);
            ok = dist2f(mx, my, mz) < 0.99f;
        }
        if (!ok) { /* 64 rejections in a row (p ~ 1e-20): fixed offset, never the atom itself */
            mx = 0.5f; my = mz = 0.f;
        }
        const float *xa = s->pos + 4 * a;
        pts[3 * p + 0] = fmaf(mx, rm, xa[0]);
        pts[3 * p + 1] = fmaf(my, rm, xa[1]);
        pts[3 * p + 2] = fmaf(mz, rm, xa[2]);
    }
}

/* ---------------------------------------------------------------------------
 * K2: field, src/isspa_force_cuda.cu:110-206.  Per point p owned by atom a:
 *   inside rmax[type(a)] (:154): count (:155); g lerped with the g-grid bin
 *   (:157-167), bin<0 => density 0 (:159-160), bin>=nGRs-1 => factor 1;
 *   mean field += r*etab/d with the same bin on the E-grid (:171-176);
 *   outside: E0 -= e0*q*r/d^3 (:179);  always E -= e0*q*r/d^3 (:183).
 * Flattened table rows: bin+1 may run into the next type's row as in the
 * reference; the caller pads each table with zeros at its end.
 * ------------------------------------------------------------------------- */
static void field_impl(const orc_isspa_sys *s, int n_mc, const float *pts, const long *idx, long count,
                       double *w, int *cnt, double *efield, double *e0field);

void orc_field(const orc_isspa_sys *s, int n_mc, const float *pts, double *w, int *cnt,
               double *efield, double *e0field) {
    field_impl(s, n_mc, pts, NULL, (long)s->n_atoms * n_mc, w, cnt, efield, e0field);
}

void orc_field_at(const orc_isspa_sys *s, int n_mc, const float *pts, const long *idx, long count,
                  double *w, int *cnt, double *efield, double *e0field) {
    field_impl(s, n_mc, pts, idx, count, w, cnt, efield, e0field);
}

/* Outputs at position q for point idx[q] (or q when idx is NULL). */
static void field_impl(const orc_isspa_sys *s, int n_mc, const float *pts, const long *idx, long count,
                       double *w, int *cnt, double *efield, double *e0field) {
    const int N = s->n_atoms;
    const float L = s->box, h = 0.5f * s->box;
    const double e0 = orc_e0();
    const float g_inv = 1.0f / s->g_dr;
#pragma omp parallel for schedule(dynamic, 64)
    for (long q = 0; q < count; ++q) {
        const long p = idx ? idx[q] : q;
        const int a = (int)(p / n_mc);
        const float rm = s->rmax[s->isspa_type[a]];
        const float rm2 = rm * rm;
        const float px = pts[3 * p], py = pts[3 * p + 1], pz = pts[3 * p + 2];
        double wp = 1.0, E[3] = {0, 0, 0}, E0[3] = {0, 0, 0};
        int n = 0;
        for (int j = 0; j < N; ++j) {
            const float *xj = s->pos + 4 * j;
            const float rx = mimg(px - xj[0], L, h);
            const float ry = mimg(py - xj[1], L, h);
            const float rz = mimg(pz - xj[2], L, h);
            const float d2 = dist2f(rx, ry, rz);
            const double dx = rx, dy = ry, dz = rz;
            const double dd = sqrt(dx * dx + dy * dy + dz * dz);
            const double c = e0 * (double)xj[3] / (dd * dd * dd);
            E[0] -= c * dx; E[1] -= c * dy; E[2] -= c * dz;
            if (d2 <= rm2) {
                ++n;
                const float dist = sqrtf(d2);
                const int bin = (int)((dist - s->g_r0) * g_inv);
                const int jt = s->isspa_type[j];
                if (bin < 0) {
                    wp = 0.0;
                } else if (bin < s->n_g - 1) {
                    double fr = (dd - ((double)s->g_r0 + bin * (double)s->g_dr)) / s->g_dr;
                    long gi = (long)jt * s->n_g + bin;
                    wp *= s->g_table[gi] * (1.0 - fr) + s->g_table[gi + 1] * fr;
                    double fe = (dd - ((double)s->e_r0 + bin * (double)s->e_dr)) / s->e_dr;
                    long ei = (long)jt * s->n_e + bin;
                    double et = s->e_table[ei] * (1.0 - fe) + s->e_table[ei + 1] * fe;
                    E[0] += dx * et / dd; E[1] += dy * et / dd; E[2] += dz * et / dd;
                }
            } else {
                E0[0] -= c * dx; E0[1] -= c * dy; E0[2] -= c * dz;
            }
        }
        w[q] = wp;
        cnt[q] = n;
        for (int k = 0; k < 3; ++k) {
            efield[3 * q + k] = E[k];
            e0field[3 * q + k] = E0[k];
        }
    }
}

/* Langevin averages for a dipole in field x: <P1>=coth x-1/x (c1 of
 * isspa_force_cuda.cu:271), <P2>=1.5*c2-0.5 (:283), <P3>=2.5*c3-1.5*c1 (:287).
 * The closed forms cancel catastrophically as x->0.  These averages are the
 * ratios i_l(x)/i_0(x) of modified spherical Bessel functions; below 5 they
 * are evaluated from the backward continued fraction of i_l/i_(l-1),
 * r_l = x / (2l+1 + x r_(l+1)), whose terms are all positive. */
static int g_langevin_float_closed = 0;

/* Diagnostic mode: evaluate the averages as the reference does, with its closed
 * forms in float (isspa_force_cuda.cu:270-273), to measure what their
 * cancellation does to the mean force. */
void orc_set_langevin_mode(int float_closed_forms) { g_langevin_float_closed = float_closed_forms; }

void orc_langevin(double x, double out[3]) {
    if (g_langevin_float_closed) {
        const float xf = (float)x;
        const float cothE = 1.0f / tanhf(xf);
        const float c1 = cothE - 1.0f / xf;
        const float c2 = 1.0f - 2.0f * (c1 / xf);
        const float c3 = cothE - 3.0f * (c2 / xf);
        out[0] = c1;
        out[1] = 1.5f * c2 - 0.5f;
        out[2] = 2.5f * c3 - 1.5f * c1;
        return;
    }
    if (x < 5.0) {
        double r = 0.0, r2 = 0.0, r3 = 0.0;
        for (int l = 40; l >= 1; --l) {
            r = x / ((double)(2 * l + 1) + x * r);
            if (l == 3) r3 = r;
            if (l == 2) r2 = r;
        }
        out[0] = r;
        out[1] = r * r2;
        out[2] = r * r2 * r3;
        return;
    }
    const double coth = 1.0 / tanh(x);
    const double c1 = coth - 1.0 / x;
    const double c2 = 1.0 - 2.0 * c1 / x;
    const double c3 = coth - 3.0 * c2 / x;
    out[0] = c1;
    out[1] = 1.5 * c2 - 0.5;
    out[2] = 2.5 * c3 - 1.5 * c1;
}

/* ---------------------------------------------------------------------------
 * K3: force, src/isspa_force_cuda.cu:208-327.  For atom i and every point p:
 *   rho = w_p * vtot[type i] / n_p (:253-254); unit field and |E| (:256-260);
 *   E0/3 (:261-263); multipole force (:270-289); inside rmax[type i]: tabulated
 *   mean LJ force with nearest-bin index and lerp (:291-305), bin>=nRs => 0
 *   (:293-294); outside: constant-density dielectric (:306-312).
 * A zero field (|E| == 0) contributes no multipole force (the reference
 * divides 0/0 there).
 * ------------------------------------------------------------------------- */
static void force_impl(const orc_isspa_sys *s, int n_mc, const float *pts, const double *w, const int *cnt,
                       const double *efield, const double *e0field, int term_mask, const int *atoms,
                       int n_sel, double *f);

void orc_isspa_force(const orc_isspa_sys *s, int n_mc, const float *pts, const double *w,
                     const int *cnt, const double *efield, const double *e0field,
                     int term_mask, double *f) {
    force_impl(s, n_mc, pts, w, cnt, efield, e0field, term_mask, NULL, s->n_atoms, f);
}

void orc_isspa_force_atoms(const orc_isspa_sys *s, int n_mc, const float *pts, const double *w,
                           const int *cnt, const double *efield, const double *e0field, int term_mask,
                           const int *atoms, int n_sel, double *f) {
    force_impl(s, n_mc, pts, w, cnt, efield, e0field, term_mask, atoms, n_sel, f);
}

/* Force on atoms[ii] (or ii when atoms is NULL) accumulated into f[ii]. */
static void force_impl(const orc_isspa_sys *s, int n_mc, const float *pts, const double *w, const int *cnt,
                       const double *efield, const double *e0field, int term_mask, const int *atoms,
                       int n_sel, double *f) {
    const int N = s->n_atoms;
    const long P = (long)N * n_mc;
    const float L = s->box, h = 0.5f * s->box;
    const float f_inv = 1.0f / s->f_dr;
    const double p0 = ORC_P0, q0 = ORC_Q0, o0 = ORC_O0;
    /* per-point prologue, computed once per point */
    double *pp = (double *)malloc(sizeof(double) * 12 * (size_t)(P > 0 ? P : 1));
#pragma omp parallel for schedule(static)
    for (long p = 0; p < P; ++p) {
        double *q = pp + 12 * p;
        const double *E = efield + 3 * p;
        const double mag = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
        double lg[3];
        orc_langevin(mag, lg);
        const double inv_n = 1.0 / cnt[p];
        q[0] = w[p] * inv_n; /* density per unit vtot */
        q[1] = inv_n;
        if (mag > 0) {
            q[2] = E[0] / mag; q[3] = E[1] / mag; q[4] = E[2] / mag;
        } else {
            q[2] = q[3] = q[4] = 0.0;
        }
        q[5] = lg[0]; q[6] = lg[1]; q[7] = lg[2];
        q[8] = e0field[3 * p] / 3.0; q[9] = e0field[3 * p + 1] / 3.0; q[10] = e0field[3 * p + 2] / 3.0;
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int ii = 0; ii < n_sel; ++ii) {
        const int i = atoms ? atoms[ii] : ii;
        const float *xi = s->pos + 4 * i;
        const int it = s->isspa_type[i];
        const float rm = s->rmax[it];
        const float rm2 = rm * rm;
        const double vt = s->vtot[it];
        const double qi = xi[3];
        double F[3] = {0, 0, 0};
        for (long p = 0; p < P; ++p) {
            const double *q = pp + 12 * p;
            const float rx = mimg(pts[3 * p] - xi[0], L, h);
            const float ry = mimg(pts[3 * p + 1] - xi[1], L, h);
            const float rz = mimg(pts[3 * p + 2] - xi[2], L, h);
            const float d2 = dist2f(rx, ry, rz);
            const double dx = rx, dy = ry, dz = rz;
            const double dd2 = dx * dx + dy * dy + dz * dz;
            const double dd = sqrt(dd2);
            const double rho = q[0] * vt;
            if (term_mask & ORC_ISSPA_MULTIPOLE) {
                const double ex = q[2], ey = q[3], ez = q[4];
                const double Rz = (ex * dx + ey * dy + ez * dz) / dd;
                const double dp1 = 3.0 * Rz;
                const double dp2 = 7.5 * Rz * Rz - 1.5;
                const double dp3 = (17.5 * Rz * Rz - 7.5) * Rz;
                double fs = -qi * p0 * q[5] * rho / (dd2 * dd);
                F[0] += fs * (dx * dp1 / dd - ex);
                F[1] += fs * (dy * dp1 / dd - ey);
                F[2] += fs * (dz * dp1 / dd - ez);
                fs = -qi * q0 * q[6] * rho / (dd2 * dd2);
                F[0] += fs * (dx * dp2 / dd - dp1 * ex);
                F[1] += fs * (dy * dp2 / dd - dp1 * ey);
                F[2] += fs * (dz * dp2 / dd - dp1 * ez);
                fs = -qi * o0 * q[7] * rho / (dd2 * dd2 * dd);
                F[0] += fs * (dx * dp3 / dd - dp2 * ex);
                F[1] += fs * (dy * dp3 / dd - dp2 * ey);
                F[2] += fs * (dz * dp3 / dd - dp2 * ez);
            }
            if (d2 <= rm2) {
                if (term_mask & ORC_ISSPA_LJ) {
                    const float dist = sqrtf(d2);
                    const int bin = (int)fmaf(dist - s->f_r0, f_inv, 0.5f);
                    double fs = 0.0;
                    if (bin >= 0 && bin < s->n_f) {
                        const double fr = (dd - ((double)s->f_r0 + bin * (double)s->f_dr)) / s->f_dr;
                        const long fi = (long)it * s->n_f + bin;
                        fs = (s->f_table[fi] * (1.0 - fr) + s->f_table[fi + 1] * fr) * rho;
                    }
                    F[0] -= dx * fs / dd; F[1] -= dy * fs / dd; F[2] -= dz * fs / dd;
                }
            } else if (term_mask & ORC_ISSPA_CDD) {
                const double igo = vt * q[1];
                const double fs = -qi * p0 / (dd2 * dd);
                const double pdr = 3.0 * (q[8] * dx + q[9] * dy + q[10] * dz) / dd2;
                F[0] += fs * (pdr * dx - q[8]) * igo;
                F[1] += fs * (pdr * dy - q[9]) * igo;
                F[2] += fs * (pdr * dz - q[10]) * igo;
            }
        }
        f[3 * ii] += F[0]; f[3 * ii + 1] += F[1]; f[3 * ii + 2] += F[2];
    }
    free(pp);
}

/* Exclusion test with the reference's ascending-list scan semantics
 * (nonbond_force_cuda.cu:72-108): the lower-index atom's list is walked in
 * order and the scan stops at the first entry larger than the partner. */
static int orc_excluded(const orc_nb_sys *s, int i, int j) {
    int a = i < j ? i : j, b = i < j ? j : i;
    if (a == b) return 0;
    int start = a == 0 ? 0 : s->n_excl_cum[a - 1];
    int stop = s->n_excl_cum[a];
    for (int e = start; e < stop; ++e) {
        if (s->excl_list[e] == b) return 1;
        if (s->excl_list[e] > b) return 0;
    }
    return 0;
}

/* ---------------------------------------------------------------------------
 * K4: nonbond, src/nonbond_force_cuda.cu:31-174.  Non-excluded pairs: LJ
 * r^-6(12A r^-6 - 6B)/r^2 (:131-132) + Coulomb q1q2/r^3 (:136) + correction;
 * excluded pairs: correction only (:153-162).  Correction (:141-147): r >
 * 2 rmax[type j] => -2q1q2(1-1/ep)/(3r^3), else -q1q2(1-1/ep)(8rmax-3r)/(24
 * rmax^4).  Force on atom i only.  With s->cut2 > 0 (the engine's optional
 * cutoff mode, not on the reference's live path) a pair counts only when its
 * FP32 squared minimum-image distance is below cut2: all three terms
 * truncated there, no shift.
 * ------------------------------------------------------------------------- */
static void nonbond_impl(const orc_nb_sys *s, int term_mask, const int *atoms, int n_sel, double *f);

void orc_nonbond(const orc_nb_sys *s, int term_mask, double *f) { nonbond_impl(s, term_mask, NULL, s->n_atoms, f); }

void orc_nonbond_atoms(const orc_nb_sys *s, int term_mask, const int *atoms, int n_sel, double *f) {
    nonbond_impl(s, term_mask, atoms, n_sel, f);
}

/* Force on atoms[ii] (or ii when atoms is NULL) accumulated into f[ii]. */
static void nonbond_impl(const orc_nb_sys *s, int term_mask, const int *atoms, int n_sel, double *f) {
    const int N = s->n_atoms;
    const float L = s->box, h = 0.5f * s->box;
    const double epf = 1.0 - 1.0 / (double)ORC_EP;
#pragma omp parallel for schedule(dynamic, 4)
    for (int ii = 0; ii < n_sel; ++ii) {
        const int i = atoms ? atoms[ii] : ii;
        const float *xi = s->pos + 4 * i;
        double F[3] = {0, 0, 0};
        for (int j = 0; j < N; ++j) {
            if (j == i) continue;
            const float *xj = s->pos + 4 * j;
            const float rx = mimg(xi[0] - xj[0], L, h);
            const float ry = mimg(xi[1] - xj[1], L, h);
            const float rz = mimg(xi[2] - xj[2], L, h);
            const float d2 = dist2f(rx, ry, rz);
            if (s->cut2 > 0.0f && !(d2 < s->cut2)) continue;
            const double dx = rx, dy = ry, dz = rz;
            const double dd2 = dx * dx + dy * dy + dz * dz;
            const double dd = sqrt(dd2);
            const double qq = (double)xi[3] * (double)xj[3];
            const float rmj = s->rmax[s->isspa_type[j]];
            const float two = 2.0f * rmj;
            double fs = 0.0;
            if (term_mask & ORC_NB_CORR) {
                if (d2 > two * two) {
                    fs += -2.0 * qq * epf / (3.0 * dd2 * dd);
                } else {
                    const double r4 = (double)rmj * rmj * rmj * rmj;
                    fs += -qq * epf * (8.0 * rmj - 3.0 * dd) / (24.0 * r4);
                }
            }
            if (!orc_excluded(s, i, j)) {
                if (term_mask & ORC_NB_LJ) {
                    const int nlj = s->nb_parm_index[s->n_types * s->lj_type[i] + s->lj_type[j]];
                    const double A = s->lj_ab[2 * nlj], B = s->lj_ab[2 * nlj + 1];
                    const double r6 = 1.0 / (dd2 * dd2 * dd2);
                    fs += r6 * (12.0 * A * r6 - 6.0 * B) / dd2;
                }
                if (term_mask & ORC_NB_COUL) fs += qq / (dd2 * dd);
            }
            F[0] += fs * dx; F[1] += fs * dy; F[2] += fs * dz;
        }
        f[3 * ii] += F[0]; f[3 * ii + 1] += F[1]; f[3 * ii + 2] += F[2];
    }
}

static inline void rvec(const float *pos, int a, int b, float L, float h, double r[3]) {
    r[0] = mimg(pos[4 * a] - pos[4 * b], L, h);
    r[1] = mimg(pos[4 * a + 1] - pos[4 * b + 1], L, h);
    r[2] = mimg(pos[4 * a + 2] - pos[4 * b + 2], L, h);
}

/* K5: bond, src/bond_force_cuda.cu:36-50: f = 2k(r0/|r| - 1) r on atom x. */
void orc_bonds(int nb, const int *atoms, const float *params, const float *pos, float box,
               double *f) {
    const float L = box, h = 0.5f * box;
    for (int b = 0; b < nb; ++b) {
        int x = atoms[3 * b], y = atoms[3 * b + 1], t = atoms[3 * b + 2];
        double r[3];
        rvec(pos, x, y, L, h, r);
        double d = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        double fb = params[2 * t] * (params[2 * t + 1] / d - 1.0);
        for (int k = 0; k < 3; ++k) {
            f[3 * x + k] += fb * r[k];
            f[3 * y + k] -= fb * r[k];
        }
    }
}

/* K6: angle, src/angle_force_cuda.cu:19-52. */
void orc_angles(int na, const int *atoms, const float *params, const float *pos, float box,
                double *f) {
    const float L = box, h = 0.5f * box;
    for (int a = 0; a < na; ++a) {
        int x = atoms[4 * a], y = atoms[4 * a + 1], z = atoms[4 * a + 2], t = atoms[4 * a + 3];
        double r1[3], r2[3];
        rvec(pos, x, y, L, h, r1);
        rvec(pos, y, z, L, h, r2);
        double c11 = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
        double c22 = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
        double c12 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
        double b = -c12 / sqrt(c11 * c22);
        double theta = b >= 1.0 ? 1.0e-16 : (b <= -1.0 ? (double)ORC_PI : acos(b));
        double fa = params[2 * t] * (theta - params[2 * t + 1]) / sqrt(c11 * c22 - c12 * c12);
        for (int k = 0; k < 3; ++k) {
            f[3 * x + k] += fa * (c12 / c11 * r1[k] - r2[k]);
            f[3 * y + k] += fa * ((1.0 + c12 / c22) * r2[k] - (1.0 + c12 / c11) * r1[k]);
            f[3 * z + k] += fa * (r1[k] - c12 / c22 * r2[k]);
        }
    }
}

/* K7: dihedral + scaled 1-4, src/dih_force_cuda.cu:48-135. */
void orc_dihedrals(int nd, const int *atoms, const int *types, const float *params,
                   const float *scaled14, const int *lj_type, const int *nb_parm_index,
                   int n_types, const double *lj_ab, const float *pos, float box,
                   int with_14, double *f) {
    const float L = box, h = 0.5f * box;
    for (int d = 0; d < nd; ++d) {
        int ax = atoms[4 * d], ay = atoms[4 * d + 1], az = atoms[4 * d + 2], aw = atoms[4 * d + 3];
        int t = types[d];
        if (with_14 && az > 0 && aw > 0) { /* :60 */
            int nlj = nb_parm_index[n_types * lj_type[ax] + lj_type[aw]];
            double A = lj_ab[2 * nlj], B = lj_ab[2 * nlj + 1];
            double r14[3];
            rvec(pos, ax, aw, L, h, r14);
            double rm = r14[0] * r14[0] + r14[1] * r14[1] + r14[2] * r14[2];
            double r6 = 1.0 / (rm * rm * rm);
            double fe = (double)pos[4 * ax + 3] * pos[4 * aw + 3] / (rm * sqrt(rm) * scaled14[2 * t]);
            double fv = r6 * (12.0 * A * r6 - 6.0 * B) / (scaled14[2 * t + 1] * rm);
            for (int k = 0; k < 3; ++k) {
                f[3 * ax + k] += (fe + fv) * r14[k];
                f[3 * aw + k] -= (fe + fv) * r14[k];
            }
        }
        if (aw < 0) aw = -aw;
        if (az < 0) az = -az;
        double r12[3], r23[3], r34[3];
        rvec(pos, ax, ay, L, h, r12);
        rvec(pos, ay, az, L, h, r23);
        rvec(pos, az, aw, L, h, r34);
        double c11 = r12[0] * r12[0] + r12[1] * r12[1] + r12[2] * r12[2];
        double c22 = r23[0] * r23[0] + r23[1] * r23[1] + r23[2] * r23[2];
        double c12 = r12[0] * r23[0] + r12[1] * r23[1] + r12[2] * r23[2];
        double c33 = r34[0] * r34[0] + r34[1] * r34[1] + r34[2] * r34[2];
        double c23 = r23[0] * r34[0] + r23[1] * r34[1] + r23[2] * r34[2];
        double c13 = r12[0] * r34[0] + r12[1] * r34[1] + r12[2] * r34[2];
        double t1 = c13 * c22 - c12 * c23;
        double t2 = c11 * c23 - c12 * c13;
        double t3 = c12 * c12 - c11 * c22;
        double t4 = c22 * c33 - c23 * c23;
        double t5 = c13 * c23 - c12 * c33;
        double t6 = -t1;
        double b = sqrt(-t3 * t4);
        double a = t6 / b;
        double fd = 0.0;
        if (a > -1.0 && a < 1.0) {
            double phi = acos(a);
            const float *pr = params + 4 * t;
            fd = pr[0] * pr[1] * sin(pr[0] * phi - pr[2]) * c22 / (sin(phi) * b);
        }
        for (int k = 0; k < 3; ++k) {
            double f1 = fd / t3 * (t1 * r12[k] + t2 * r23[k] + t3 * r34[k]);
            double f4 = -fd / t4 * (t4 * r12[k] + t5 * r23[k] + t6 * r34[k]);
            f[3 * ax + k] += f1;
            f[3 * ay + k] += -(1.0 + c12 / c22) * f1 + c23 / c22 * f4;
            f[3 * az + k] += c12 / c22 * f1 - (1.0 + c23 / c22) * f4;
            f[3 * aw + k] += f4;
        }
    }
}

/* K9: umbrella, src/us_force_cuda.cu:14-48 with kumb = [-k, +k]
 * (us_class.cpp:153-154).  COM from wrapped positions, mass fractions. */
void orc_us(int nbias, const int *list, const float *mfrac, double k, double x0,
            const float *pos, float box, double *f, double *com) {
    double c[2][3] = {{0, 0, 0}, {0, 0, 0}};
    for (int b = 0; b < nbias; ++b) {
        int a = list[2 * b], g = list[2 * b + 1];
        for (int d = 0; d < 3; ++d) c[g][d] += (double)mfrac[b] * pos[4 * a + d];
    }
    double L = box, h = 0.5 * box, r[3];
    for (int d = 0; d < 3; ++d) {
        r[d] = c[0][d] - c[1][d];
        if (r[d] > h) r[d] -= L;
        else if (r[d] < -h) r[d] += L;
    }
    double dist = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (int b = 0; b < nbias; ++b) {
        int a = list[2 * b], g = list[2 * b + 1];
        double ku = g == 0 ? -k : k;
        double pf = ku * (dist - x0) * mfrac[b] / dist;
        for (int d = 0; d < 3; ++d) f[3 * a + d] += pf * r[d];
    }
    if (com)
        for (int g = 0; g < 2; ++g)
            for (int d = 0; d < 3; ++d) com[3 * g + d] = c[g][d];
}

/* K8: leapfrog + Andersen, src/leapfrog_cuda.cu:44-64.  Random numbers come
 * from Philox stream 1 keyed by (seed, step, window, atom). */
void orc_leapfrog(int n, const float *pos, const float *vel, const double *f, float kT,
                  float dt, float pnu, float box, uint64_t seed, uint32_t step,
                  uint32_t window, double *pos_out, double *vel_out, int *resampled) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int i = 0; i < n; ++i) {
        uint32_t c0[4] = {(uint32_t)i, 0u, step, (window << 8) | 1u}, o0[4];
        orc_philox4x32_10(c0, key, o0);
        const float u = u24(o0[0]);
        const double m = vel[4 * i + 3];
        double v[3], x[3];
        int res = u < pnu;
        if (res) {
            uint32_t c1[4] = {(uint32_t)i, 1u, step, (window << 8) | 1u}, o1[4];
            orc_philox4x32_10(c1, key, o1);
            const double twopi = 6.283185307179586;
            double ra = sqrt(-2.0 * log(u24open(o1[0]))), rb = sqrt(-2.0 * log(u24open(o1[2])));
            double nrm[3] = {ra * cos(twopi * u24open(o1[1])), ra * sin(twopi * u24open(o1[1])),
                             rb * cos(twopi * u24open(o1[3]))};
            double sd = sqrt((double)kT / m);
            for (int d = 0; d < 3; ++d) v[d] = nrm[d] * sd + f[3 * i + d] * dt / (2.0 * m);
        } else {
            for (int d = 0; d < 3; ++d) v[d] = vel[4 * i + d] + f[3 * i + d] * dt / m;
        }
        for (int d = 0; d < 3; ++d) {
            x[d] = pos[4 * i + d] + v[d] * dt;
            if (x[d] > box) x[d] -= box;
            else if (x[d] < 0.0) x[d] += box;
            pos_out[3 * i + d] = x[d];
            vel_out[3 * i + d] = v[d];
        }
        if (resampled) resampled[i] = res;
    }
}

static int cmp_int(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* K10: neighbour list, src/neighborlist_cuda.cu:37-96: every ordered pair
 * atom1 != atom2, not excluded, with r^2 < rNN^2.  The reference appends in
 * atomic order; the oracle returns each row sorted. */
long orc_neighbor_list(const orc_nb_sys *s, float rnn2, int max_per_atom, int *rows,
                       int *counts) {
    const int N = s->n_atoms;
    const float L = s->box, h = 0.5f * s->box;
    long total = 0;
    for (int i = 0; i < N; ++i) {
        int c = 0;
        for (int j = 0; j < N; ++j) {
            if (j == i || orc_excluded(s, i, j)) continue;
            const float *xi = s->pos + 4 * i, *xj = s->pos + 4 * j;
            float rx = mimg(xi[0] - xj[0], L, h), ry = mimg(xi[1] - xj[1], L, h),
                  rz = mimg(xi[2] - xj[2], L, h);
            if (dist2f(rx, ry, rz) < rnn2) {
                if (c < max_per_atom) rows[(long)i * max_per_atom + c] = j;
                ++c;
            }
        }
        int m = c < max_per_atom ? c : max_per_atom;
        qsort(rows + (long)i * max_per_atom, (size_t)m, sizeof(int), cmp_int);
        counts[i] = c;
        total += c;
    }
    return total;
}

/* K11: cell index, src/cell_list_cuda.cu:27-29. */
void orc_cell_index(int n, const float *pos, float rc, const int ncell[3], int *cell) {
    for (int i = 0; i < n; ++i) {
        int cx = (int)(pos[4 * i] / rc), cy = (int)(pos[4 * i + 1] / rc), cz = (int)(pos[4 * i + 2] / rc);
        cell[i] = cx * ncell[1] * ncell[2] + cy * ncell[2] + cz;
    }
}

/* ---------------------------------------------------------------------------
 * Adjoint of J = sum_i c_i . F_i for one frame, in FP64 (naive reference
 * gradient).  Writing the IS-SPA force of point p on atom i as
 *   F_ip = s_p G_ip + H_ip,   s_p = w_p / n_p,
 * with G the multipole and tabulated-LJ parts per unit density and H the
 * constant-density-dielectric part (isspa_force_cuda.cu:274-312), the
 * derivatives are
 *   dJ/ds_p        = sum_i c_i . G_ip                       (lambda_p)
 *   dJ/dT_f[k]     = sum_{i,p} c_i . (-vtot_i s_p r/d) * lerp weight of k
 *   dJ/dT_g[k]     = sum_p lambda_p / n_p * dw_p/dT_g[k],  w_p = prod_j g_j
 * and, for the nonbond LJ (nonbond_force_cuda.cu:131-132) and the scaled 1-4
 * LJ (dih_force_cuda.cu:70-74), the coefficients enter linearly.
 * ------------------------------------------------------------------------- */
double orc_adjoint(const orc_isspa_sys *s, const orc_nb_sys *nb, int n_mc, const float *pts,
                   const double *c, int nd, const int *dih_atoms, const int *dih_types,
                   const float *scaled14, double *dJ_df, double *dJ_dg, double *dJ_dA,
                   double *dJ_dB) {
    const int N = s->n_atoms;
    const long P = (long)N * n_mc;
    const float L = s->box, h = 0.5f * s->box;
    const double p0 = ORC_P0, q0 = ORC_Q0, o0 = ORC_O0;
    double *w = (double *)malloc(sizeof(double) * (size_t)P);
    int *cnt = (int *)malloc(sizeof(int) * (size_t)P);
    double *E = (double *)malloc(sizeof(double) * 3 * (size_t)P);
    double *E0 = (double *)malloc(sizeof(double) * 3 * (size_t)P);
    double *lam = (double *)calloc((size_t)P, sizeof(double));
    orc_field(s, n_mc, pts, w, cnt, E, E0);
    const float f_inv = 1.0f / s->f_dr, g_inv = 1.0f / s->g_dr;
    const long nF = (long)s->n_itypes * s->n_f, nG = (long)s->n_itypes * s->n_g;
    double J = 0.0;
    /* IS-SPA force part: value, lambda_p, force-table adjoint */
    for (long p = 0; p < P; ++p) {
        const double *Ep = E + 3 * p;
        const double mag = sqrt(Ep[0] * Ep[0] + Ep[1] * Ep[1] + Ep[2] * Ep[2]);
        double lg[3];
        orc_langevin(mag, lg);
        const double eh[3] = {mag > 0 ? Ep[0] / mag : 0, mag > 0 ? Ep[1] / mag : 0, mag > 0 ? Ep[2] / mag : 0};
        const double inv_n = 1.0 / cnt[p], sp = w[p] * inv_n;
        const double e03[3] = {E0[3 * p] / 3.0, E0[3 * p + 1] / 3.0, E0[3 * p + 2] / 3.0};
        for (int i = 0; i < N; ++i) {
            const double *ci = c + 3 * i;
            if (ci[0] == 0.0 && ci[1] == 0.0 && ci[2] == 0.0) continue;
            const float *xi = s->pos + 4 * i;
            const int it = s->isspa_type[i];
            const float rm = s->rmax[it];
            const double vt = s->vtot[it], qi = xi[3];
            const float rx = mimg(pts[3 * p] - xi[0], L, h), ry = mimg(pts[3 * p + 1] - xi[1], L, h),
                        rz = mimg(pts[3 * p + 2] - xi[2], L, h);
            const float d2 = dist2f(rx, ry, rz);
            const double r[3] = {rx, ry, rz};
            const double dd2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2], dd = sqrt(dd2);
            const double Rz = (eh[0] * r[0] + eh[1] * r[1] + eh[2] * r[2]) / dd;
            const double dp1 = 3.0 * Rz, dp2 = 7.5 * Rz * Rz - 1.5, dp3 = (17.5 * Rz * Rz - 7.5) * Rz;
            const double t1 = p0 * lg[0] / (dd2 * dd), t2 = q0 * lg[1] / (dd2 * dd2), t3 = o0 * lg[2] / (dd2 * dd2 * dd);
            double G[3], H[3] = {0, 0, 0};
            for (int k = 0; k < 3; ++k) {
                const double mu = t1 * (r[k] * dp1 / dd - eh[k]) + t2 * (r[k] * dp2 / dd - dp1 * eh[k]) +
                                  t3 * (r[k] * dp3 / dd - dp2 * eh[k]);
                G[k] = -qi * vt * mu;
            }
            if (d2 <= rm * rm) {
                const float dist = sqrtf(d2);
                const int bin = (int)fmaf(dist - s->f_r0, f_inv, 0.5f);
                if (bin >= 0 && bin < s->n_f) {
                    const double fr = (dd - ((double)s->f_r0 + bin * (double)s->f_dr)) / s->f_dr;
                    const long fi = (long)it * s->n_f + bin;
                    const double tab = s->f_table[fi] * (1.0 - fr) + s->f_table[fi + 1] * fr;
                    double cr = 0.0;
                    for (int k = 0; k < 3; ++k) {
                        G[k] += -vt * tab * r[k] / dd;
                        cr += ci[k] * (-vt * sp * r[k] / dd);
                    }
                    dJ_df[fi] += cr * (1.0 - fr);
                    if (fi + 1 < nF) dJ_df[fi + 1] += cr * fr;
                }
            } else {
                const double fs = -qi * p0 / (dd2 * dd);
                const double pdr = 3.0 * (e03[0] * r[0] + e03[1] * r[1] + e03[2] * r[2]) / dd2;
                for (int k = 0; k < 3; ++k) H[k] = fs * (pdr * r[k] - e03[k]) * vt * inv_n;
            }
            for (int k = 0; k < 3; ++k) {
                J += ci[k] * (sp * G[k] + H[k]);
                lam[p] += ci[k] * G[k];
            }
        }
    }
    /* density-table adjoint through w_p = prod_j g_j (isspa_force_cuda.cu:157-167) */
    for (long p = 0; p < P; ++p) {
        if (lam[p] == 0.0) continue;
        const int a = (int)(p / n_mc);
        const float rm = s->rmax[s->isspa_type[a]];
        const double dJdw = lam[p] / cnt[p];
        int zeros = 0, forced_zero = 0;
        double prod_nz = 1.0;
        for (int pass = 0; pass < 2; ++pass) {
            for (int j = 0; j < N; ++j) {
                const float *xj = s->pos + 4 * j;
                const float rx = mimg(pts[3 * p] - xj[0], L, h), ry = mimg(pts[3 * p + 1] - xj[1], L, h),
                            rz = mimg(pts[3 * p + 2] - xj[2], L, h);
                const float d2 = dist2f(rx, ry, rz);
                if (!(d2 <= rm * rm)) continue;
                const float dist = sqrtf(d2);
                const int bin = (int)((dist - s->g_r0) * g_inv);
                if (bin < 0) {
                    forced_zero = 1;
                    continue;
                }
                if (bin >= s->n_g - 1) continue;
                const double dd = sqrt((double)rx * rx + (double)ry * ry + (double)rz * rz);
                const double fr = (dd - ((double)s->g_r0 + bin * (double)s->g_dr)) / s->g_dr;
                const long gi = (long)s->isspa_type[j] * s->n_g + bin;
                const double g = s->g_table[gi] * (1.0 - fr) + s->g_table[gi + 1] * fr;
                if (pass == 0) {
                    if (g == 0.0) ++zeros;
                    else prod_nz *= g;
                } else {
                    double others;
                    if (forced_zero || zeros >= 2) others = 0.0;
                    else if (zeros == 1) others = g == 0.0 ? prod_nz : 0.0;
                    else others = prod_nz / g;
                    const double d = dJdw * others;
                    dJ_dg[gi] += d * (1.0 - fr);
                    if (gi + 1 < nG) dJ_dg[gi + 1] += d * fr;
                }
            }
        }
    }
    /* nonbond: value and LJ coefficient adjoint (nonbond_force_cuda.cu:123-162) */
    {
        const double epf = 1.0 - 1.0 / (double)ORC_EP;
        for (int i = 0; i < N; ++i) {
            const double *ci = c + 3 * i;
            if (ci[0] == 0.0 && ci[1] == 0.0 && ci[2] == 0.0) continue;
            const float *xi = nb->pos + 4 * i;
            for (int j = 0; j < N; ++j) {
                if (j == i) continue;
                const float *xj = nb->pos + 4 * j;
                const float rx = mimg(xi[0] - xj[0], L, h), ry = mimg(xi[1] - xj[1], L, h), rz = mimg(xi[2] - xj[2], L, h);
                const float d2 = dist2f(rx, ry, rz);
                const double r[3] = {rx, ry, rz};
                const double dd2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2], dd = sqrt(dd2);
                const double qq = (double)xi[3] * xj[3];
                const float rmj = nb->rmax[nb->isspa_type[j]];
                const float two = 2.0f * rmj;
                double fs = d2 > two * two ? -2.0 * qq * epf / (3.0 * dd2 * dd)
                                           : -qq * epf * (8.0 * rmj - 3.0 * dd) / (24.0 * (double)rmj * rmj * rmj * rmj);
                const double cr = ci[0] * r[0] + ci[1] * r[1] + ci[2] * r[2];
                if (!orc_excluded(nb, i, j)) {
                    const int k = nb->nb_parm_index[nb->n_types * nb->lj_type[i] + nb->lj_type[j]];
                    const double r6 = 1.0 / (dd2 * dd2 * dd2);
                    fs += r6 * (12.0 * nb->lj_ab[2 * k] * r6 - 6.0 * nb->lj_ab[2 * k + 1]) / dd2 + qq / (dd2 * dd);
                    dJ_dA[k] += cr * 12.0 * r6 * r6 / dd2;
                    dJ_dB[k] += cr * (-6.0) * r6 / dd2;
                }
                J += cr * fs;
            }
        }
    }
    /* scaled 1-4 terms of the dihedrals (dih_force_cuda.cu:60-82) */
    for (int d = 0; d < nd; ++d) {
        const int ax = dih_atoms[4 * d], az = dih_atoms[4 * d + 2], aw = dih_atoms[4 * d + 3];
        if (!(az > 0 && aw > 0)) continue;
        const double *cx = c + 3 * ax, *cw = c + 3 * aw;
        const double dc[3] = {cx[0] - cw[0], cx[1] - cw[1], cx[2] - cw[2]};
        if (dc[0] == 0.0 && dc[1] == 0.0 && dc[2] == 0.0) continue;
        const int t = dih_types[d];
        const int k = nb->nb_parm_index[nb->n_types * nb->lj_type[ax] + nb->lj_type[aw]];
        double r14[3];
        rvec(nb->pos, ax, aw, L, h, r14);
        const double rm = r14[0] * r14[0] + r14[1] * r14[1] + r14[2] * r14[2];
        const double r6 = 1.0 / (rm * rm * rm);
        const double scee = scaled14[2 * t], scnb = scaled14[2 * t + 1];
        const double fe = (double)nb->pos[4 * ax + 3] * nb->pos[4 * aw + 3] / (rm * sqrt(rm) * scee);
        const double fv = r6 * (12.0 * nb->lj_ab[2 * k] * r6 - 6.0 * nb->lj_ab[2 * k + 1]) / (scnb * rm);
        const double cr = dc[0] * r14[0] + dc[1] * r14[1] + dc[2] * r14[2];
        J += cr * (fe + fv);
        dJ_dA[k] += cr * 12.0 * r6 * r6 / (scnb * rm);
        dJ_dB[k] += cr * (-6.0) * r6 / (scnb * rm);
    }
    free(w); free(cnt); free(E); free(E0); free(lam);
    return J;
}

/* ---------------------------------------------------------------------------
 * Energies and virial of one window (the potentials whose negative gradients
 * are the forces above), FP64 values from the float geometry:
 *   out[0], out[1]  kinetic m v^2/2 with v(t-dt/2) and with the
 *                   thermostat-free kick v + F dt/m (leapfrog_cuda.cu:57-60,
 *                   float arithmetic as the integrator);
 *   out[2..4]       bond k(r-r0)^2, angle k(theta-theta0)^2 (2k stored),
 *                   dihedral V(1+cos(n phi - phase));
 *   out[5], out[6]  scaled 1-4 LJ and Coulomb;
 *   out[7..9]       pair LJ, Coulomb, IS-SPA correction (nonbond_force_cuda.cu:
 *                   131-147; correction integrated from infinity with the
 *                   partner's rmax, ordered pairs halved);
 *   out[10]         umbrella k/2 (d - x0)^2;
 *   out[11]         virial sum r . F over those terms.
 * ------------------------------------------------------------------------- */
void orc_energies(const orc_nb_sys *s, int nb_terms, int n_bonds, const int *bond_atoms,
                  const float *bond_params, int n_angles, const int *angle_atoms,
                  const float *angle_params, int nd, const int *dih_atoms, const int *dih_types,
                  const float *dih_params, const float *scaled14, int nbias, const int *bias_list,
                  const float *mfrac, double us_k, double us_x0, const float *vel, const double *f,
                  float dt, double out[12]) {
    const int N = s->n_atoms;
    const float *pos = s->pos;
    const float L = s->box, h = 0.5f * s->box;
    const double epf = 1.0 - 1.0 / (double)ORC_EP;
    for (int k = 0; k < 12; ++k) out[k] = 0.0;
    double elj = 0.0, ec = 0.0, ecr = 0.0, vir = 0.0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : elj, ec, ecr, vir)
    for (int i = 0; i < N; ++i) {
        const float *xi = pos + 4 * i;
        for (int j = 0; j < N; ++j) {
            if (j == i) continue;
            const float *xj = pos + 4 * j;
            const float rx = mimg(xi[0] - xj[0], L, h);
            const float ry = mimg(xi[1] - xj[1], L, h);
            const float rz = mimg(xi[2] - xj[2], L, h);
            const float d2 = dist2f(rx, ry, rz);
            if (s->cut2 > 0.0f && !(d2 < s->cut2)) continue;
            const double dd2 = (double)rx * rx + (double)ry * ry + (double)rz * rz, dd = sqrt(dd2);
            const double qq = (double)xi[3] * (double)xj[3];
            const float rmj = s->rmax[s->isspa_type[j]];
            const float two = 2.0f * rmj;
            if (nb_terms & ORC_NB_CORR) {
                if (d2 > two * two) {
                    const double u = -2.0 * qq * epf / (3.0 * dd);
                    ecr += u;
                    vir += u;
                } else {
                    const double rm = rmj, r4 = rm * rm * rm * rm;
                    ecr += qq * epf * ((4.0 * rm * dd2 - dd2 * dd) / (24.0 * r4) - 2.0 / (3.0 * rm));
                    vir += -qq * epf * (8.0 * rm - 3.0 * dd) * dd2 / (24.0 * r4);
                }
            }
            if (!orc_excluded(s, i, j)) {
                if (nb_terms & ORC_NB_LJ) {
                    const int nlj = s->nb_parm_index[s->n_types * s->lj_type[i] + s->lj_type[j]];
                    const double A = s->lj_ab[2 * nlj], B = s->lj_ab[2 * nlj + 1];
                    const double r6 = 1.0 / (dd2 * dd2 * dd2);
                    elj += r6 * (A * r6 - B);
                    vir += r6 * (12.0 * A * r6 - 6.0 * B);
                }
                if (nb_terms & ORC_NB_COUL) {
                    ec += qq / dd;
                    vir += qq / dd;
                }
            }
        }
    }
    out[7] = 0.5 * elj;
    out[8] = 0.5 * ec;
    out[9] = 0.5 * ecr;
    out[11] = 0.5 * vir;
    for (int b = 0; b < n_bonds; ++b) {
        const int x = bond_atoms[3 * b], y = bond_atoms[3 * b + 1], t = bond_atoms[3 * b + 2];
        double r[3];
        rvec(pos, x, y, L, h, r);
        const double d = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]), dr = d - bond_params[2 * t + 1];
        out[2] += 0.5 * bond_params[2 * t] * dr * dr;
        out[11] += -(double)bond_params[2 * t] * dr * d;
    }
    for (int a = 0; a < n_angles; ++a) {
        const int x = angle_atoms[4 * a], y = angle_atoms[4 * a + 1], z = angle_atoms[4 * a + 2],
                  t = angle_atoms[4 * a + 3];
        double r1[3], r2[3];
        rvec(pos, x, y, L, h, r1);
        rvec(pos, y, z, L, h, r2);
        const double c11 = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
        const double c22 = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
        const double c12 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
        const double b = -c12 / sqrt(c11 * c22);
        const double theta = b >= 1.0 ? 1.0e-16 : (b <= -1.0 ? (double)ORC_PI : acos(b));
        const double dt_ = theta - angle_params[2 * t + 1];
        out[3] += 0.5 * angle_params[2 * t] * dt_ * dt_;
        const double fa = angle_params[2 * t] * dt_ / sqrt(c11 * c22 - c12 * c12);
        for (int k = 0; k < 3; ++k) {
            const double fx = fa * (c12 / c11 * r1[k] - r2[k]), fz = fa * (r1[k] - c12 / c22 * r2[k]);
            out[11] += r1[k] * fx - r2[k] * fz;
        }
    }
    for (int d = 0; d < nd; ++d) {
        int ax = dih_atoms[4 * d], ay = dih_atoms[4 * d + 1], az = dih_atoms[4 * d + 2], aw = dih_atoms[4 * d + 3];
        const int t = dih_types[d];
        if (az > 0 && aw > 0) {
            const int nlj = s->nb_parm_index[s->n_types * s->lj_type[ax] + s->lj_type[aw]];
            const double A = s->lj_ab[2 * nlj], B = s->lj_ab[2 * nlj + 1];
            double r14[3];
            rvec(pos, ax, aw, L, h, r14);
            const double rm = r14[0] * r14[0] + r14[1] * r14[1] + r14[2] * r14[2];
            const double r6 = 1.0 / (rm * rm * rm);
            const double uc = (double)pos[4 * ax + 3] * pos[4 * aw + 3] / (sqrt(rm) * scaled14[2 * t]);
            out[5] += r6 * (A * r6 - B) / scaled14[2 * t + 1];
            out[6] += uc;
            out[11] += r6 * (12.0 * A * r6 - 6.0 * B) / scaled14[2 * t + 1] + uc;
        }
        if (aw < 0) aw = -aw;
        if (az < 0) az = -az;
        double r12[3], r23[3], r34[3];
        rvec(pos, ax, ay, L, h, r12);
        rvec(pos, ay, az, L, h, r23);
        rvec(pos, az, aw, L, h, r34);
        const double c11 = r12[0] * r12[0] + r12[1] * r12[1] + r12[2] * r12[2];
        const double c22 = r23[0] * r23[0] + r23[1] * r23[1] + r23[2] * r23[2];
        const double c12 = r12[0] * r23[0] + r12[1] * r23[1] + r12[2] * r23[2];
        const double c33 = r34[0] * r34[0] + r34[1] * r34[1] + r34[2] * r34[2];
        const double c23 = r23[0] * r34[0] + r23[1] * r34[1] + r23[2] * r34[2];
        const double c13 = r12[0] * r34[0] + r12[1] * r34[1] + r12[2] * r34[2];
        const double t1 = c13 * c22 - c12 * c23, t2 = c11 * c23 - c12 * c13, t3 = c12 * c12 - c11 * c22;
        const double t4 = c22 * c33 - c23 * c23, t5 = c13 * c23 - c12 * c33, t6 = -t1;
        const double bb = sqrt(-t3 * t4), a = t6 / bb;
        const float *pr = dih_params + 4 * t;
        double fd = 0.0, phi = a <= -1.0 ? (double)ORC_PI : 0.0;
        if (a > -1.0 && a < 1.0) {
            phi = acos(a);
            fd = pr[0] * pr[1] * sin(pr[0] * phi - pr[2]) * c22 / (sin(phi) * bb);
        }
        out[4] += pr[1] * (1.0 + cos(pr[0] * phi - pr[2]));
        for (int k = 0; k < 3; ++k) {
            const double f1 = fd / t3 * (t1 * r12[k] + t2 * r23[k] + t3 * r34[k]);
            const double f4 = -fd / t4 * (t4 * r12[k] + t5 * r23[k] + t6 * r34[k]);
            const double f3 = c12 / c22 * f1 - (1.0 + c23 / c22) * f4;
            out[11] += r12[k] * f1 - r23[k] * f3 - (r23[k] + r34[k]) * f4;
        }
    }
    if (nbias > 0) {
        double com[6];
        double *fs = (double *)calloc(3 * (size_t)N, sizeof(double));
        orc_us(nbias, bias_list, mfrac, us_k, us_x0, pos, s->box, fs, com);
        free(fs);
        double r[3];
        for (int k = 0; k < 3; ++k) {
            r[k] = com[k] - com[3 + k];
            if (r[k] > 0.5 * s->box) r[k] -= s->box;
            else if (r[k] < -0.5 * s->box) r[k] += s->box;
        }
        const double dist = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]), dx = dist - us_x0;
        out[10] = 0.5 * us_k * dx * dx;
        out[11] += -us_k * dx * dist;
    }
    for (int i = 0; i < N; ++i) {
        const float m = vel[4 * i + 3], k = dt / m;
        double kb = 0.0, ka = 0.0;
        for (int d = 0; d < 3; ++d) {
            const float v = vel[4 * i + d];
            const float vp = fmaf((float)f[3 * i + d], k, v);
            kb += (double)v * v;
            ka += (double)vp * vp;
        }
        out[0] += 0.5 * (double)m * kb;
        out[1] += 0.5 * (double)m * ka;
    }
}
