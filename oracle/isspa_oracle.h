/*
 * isspa_oracle.h -- CPU oracle for the IS-SPA force/step path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * CUDA kernels of mccullaghlab/ISSPA-Force-Cuda (src/isspa_force_cuda.cu,
 * src/nonbond_force_cuda.cu, src/bond_force_cuda.cu, src/angle_force_cuda.cu,
 * src/dih_force_cuda.cu, src/leapfrog_cuda.cu, src/us_force_cuda.cu) used as
 * the checker for the GPU engine.  Only tests, the smoke check and the CPU
 * baseline of bench.py may load it; the product never links it.
 *
 * Numerics: every value is accumulated in double.  Every geometric
 * *decision* (minimum image, inside-rmax tests, table bin indices, the MC
 * rejection test) is evaluated in float with the exact operation sequence the
 * GPU kernels use (explicit fmaf, no contraction), so the oracle and the GPU
 * take identical branches and only rounding of values differs.
 *
 * Parity pins: the nonbond sub-terms are pinned to the reference's FP64 golden
 * force files (timing_tests/ADI2/10000MC/compare/ADI2.multi.frc.{LJsolu,Csolu,
 * Csolv_pair}.dat); the IS-SPA force branches are pinned statistically to the
 * reference's 1000-seed per-term frame averages (ISSPA_force_{LJsolv,Csolv,
 * Csolv_CDD}_10000.xyz); the Philox generator is pinned to the published
 * Random123 known-answer vectors.
 */
#ifndef ISSPA_ORACLE_H
#define ISSPA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* IS-SPA solvent model inputs of one system (isspa_class.h:10-67). */
typedef struct {
    int n_atoms;
    const float *pos;        /* [n_atoms][4]: x, y, z, charge/sqrt(eps) */
    const int *isspa_type;   /* [n_atoms], 0-based */
    int n_itypes;
    const float *rmax;       /* [n_itypes] */
    const float *vtot;       /* [n_itypes], isspa_class.cpp:41 */
    int n_g, n_e, n_f;       /* rows per type of the three tables */
    const double *g_table;   /* [n_itypes*n_g] (+ zero padding); values in FP64 */
    const double *e_table;   /* [n_itypes*n_e] */
    const double *f_table;   /* [n_itypes*n_f] */
    float g_r0, g_dr, e_r0, e_dr, f_r0, f_dr;
    float box;
} orc_isspa_sys;

/* Nonbond inputs (atom_class.h:22-49). */
typedef struct {
    int n_atoms;
    const float *pos;          /* [n_atoms][4] */
    int n_types;
    const int *lj_type;        /* [n_atoms] 0-based */
    const int *nb_parm_index;  /* [n_types*n_types] 0-based index into lj_ab */
    const double *lj_ab;       /* [n_types*(n_types+1)/2][2] A, B */
    const int *n_excl_cum;     /* [n_atoms] cumulative counts */
    const int *excl_list;      /* [excl_len] 0-based */
    const int *isspa_type;     /* [n_atoms] */
    const float *rmax;         /* [n_itypes] */
    float box;
    float cut2;                /* > 0: only pairs with FP32 squared distance below it count
                                  (the engine's optional cutoff mode); 0: every pair */
} orc_nb_sys;

/* Term masks, naming follows the reference's per-term golden files. */
enum {
    ORC_ISSPA_MULTIPOLE = 1, /* "Csolv": dipole+quadrupole+octupole polarisation */
    ORC_ISSPA_LJ = 2,        /* "LJsolv": tabulated mean LJ force           */
    ORC_ISSPA_CDD = 4,       /* "Csolv_CDD": constant-density dielectric    */
    ORC_NB_LJ = 1,           /* "LJsolu" */
    ORC_NB_COUL = 2,         /* "Csolu" */
    ORC_NB_CORR = 4          /* "Csolv_pair": IS-SPA long-range correction  */
};

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* MC points of one step (isspa_force_cuda.cu:73-107, Philox-keyed). */
void orc_mc_points(const orc_isspa_sys *s, int n_mc, uint64_t seed, uint32_t step,
                   uint32_t window, float *pts /* [N*n_mc][3] */);

/* Density product, count and mean fields per MC point (isspa_force_cuda.cu:110-206). */
void orc_field(const orc_isspa_sys *s, int n_mc, const float *pts, double *w, int *cnt,
               double *efield /* [P][3] */, double *e0field /* [P][3] */);

/* IS-SPA force on every atom from every MC point (isspa_force_cuda.cu:208-327). */
void orc_isspa_force(const orc_isspa_sys *s, int n_mc, const float *pts, const double *w,
                     const int *cnt, const double *efield, const double *e0field,
                     int term_mask, double *f /* [N][3], accumulated into */);

/* Subsets for large systems: fields at the listed point indices (outputs at
 * list positions), IS-SPA and nonbond forces on the listed atoms (f[k] for
 * atoms[k]), from all points / all partners. */
void orc_field_at(const orc_isspa_sys *s, int n_mc, const float *pts, const long *idx, long count,
                  double *w, int *cnt, double *efield, double *e0field);
void orc_isspa_force_atoms(const orc_isspa_sys *s, int n_mc, const float *pts, const double *w,
                           const int *cnt, const double *efield, const double *e0field, int term_mask,
                           const int *atoms, int n_sel, double *f);
void orc_nonbond_atoms(const orc_nb_sys *s, int term_mask, const int *atoms, int n_sel, double *f);

/* Langevin polarisation averages <P1>, <P2>, <P3> for field magnitude x. */
void orc_langevin(double x, double out[3]);
/* 1: evaluate them with the reference's float closed forms (diagnostic). */
void orc_set_langevin_mode(int float_closed_forms);

/* All-pairs LJ + Coulomb + IS-SPA correction (nonbond_force_cuda.cu:31-174). */
void orc_nonbond(const orc_nb_sys *s, int term_mask, double *f /* [N][3] += */);

/* Bonded terms (bond_force_cuda.cu:15-53, angle_force_cuda.cu:12-66, dih_force_cuda.cu:13-136). */
void orc_bonds(int nb, const int *atoms, const float *params, const float *pos, float box, double *f);
void orc_angles(int na, const int *atoms, const float *params, const float *pos, float box, double *f);
void orc_dihedrals(int nd, const int *atoms, const int *types, const float *params,
                   const float *scaled14, const int *lj_type, const int *nb_parm_index,
                   int n_types, const double *lj_ab, const float *pos, float box,
                   int with_14, double *f);

/* Umbrella COM restraint (us_force_cuda.cu:14-48); com_out[2][3]. */
void orc_us(int nbias, const int *list, const float *mfrac, double k, double x0,
            const float *pos, float box, double *f, double *com_out);

/* Leapfrog + Andersen (leapfrog_cuda.cu:33-68).  Reads float pos/vel, writes
 * double results. */
void orc_leapfrog(int n, const float *pos, const float *vel, const double *f, float kT,
                  float dt, float pnu, float box, uint64_t seed, uint32_t step,
                  uint32_t window, double *pos_out, double *vel_out, int *resampled);

/* Neighbour list rows (neighborlist_cuda.cu:11-137): per-atom sorted partners
 * with r^2 < rnn2, exclusions as the nonbond kernel.  Returns total count;
 * rows[atom*max_per_atom + k], counts[atom]. */
long orc_neighbor_list(const orc_nb_sys *s, float rnn2, int max_per_atom, int *rows,
                       int *counts);

/* Cell binning (cell_list_cuda.cu:13-35). cell[atom]. */
void orc_cell_index(int n, const float *pos, float rc, const int ncell[3], int *cell);

void orc_set_threads(int n);

/* Adjoint of J = sum_i c_i . F_i for one frame (naive FP64 reference gradient).
 * c: [N][3] weights (zero for atoms outside the restraint groups).  F_i is the
 * IS-SPA force on the given points plus the nonbond force plus the scaled 1-4
 * term of the dihedrals.  Accumulates into
 *   dJ_df [n_itypes*n_f]  (ISSPA_FORCES entries),
 *   dJ_dg [n_itypes*n_g]  (ISSPA_DENSITIES entries),
 *   dJ_dA, dJ_dB [n_types*(n_types+1)/2]  (packed LJ coefficients),
 * and returns J. */
double orc_adjoint(const orc_isspa_sys *s, const orc_nb_sys *nb, int n_mc, const float *pts,
                   const double *c, int nd, const int *dih_atoms, const int *dih_types,
                   const float *scaled14, double *dJ_df, double *dJ_dg, double *dJ_dA,
                   double *dJ_dB);

/* Energy components and virial of one window, FP64 (order of the engine's
 * ISSPA_E_* enum): kinetic before/after the kick, bond, angle, dihedral,
 * 1-4 LJ, 1-4 Coulomb, pair LJ, pair Coulomb, IS-SPA correction, umbrella,
 * virial.  vel [N][4] (v, mass); f [N][3] the step's total force; dt the
 * internal time step.  nbias = 0 skips the umbrella term. */
void orc_energies(const orc_nb_sys *s, int nb_terms, int n_bonds, const int *bond_atoms,
                  const float *bond_params, int n_angles, const int *angle_atoms,
                  const float *angle_params, int nd, const int *dih_atoms, const int *dih_types,
                  const float *dih_params, const float *scaled14, int nbias, const int *bias_list,
                  const float *mfrac, double us_k, double us_x0, const float *vel, const double *f,
                  float dt, double out[12]);

#ifdef __cplusplus
}
#endif
#endif
