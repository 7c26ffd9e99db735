/*
 * isspa_gb300.h -- C ABI of the GB300 IS-SPA implicit-solvent MD force engine.
 *
 * Drop-in replacement for the per-step force path of mccullaghlab/ISSPA-Force-
 * Cuda's total_force_cuda.x (src/total_force_cuda.cpp:102-154).  The reference
 * binds C++ class references (atom&, isspa&, bond&, ...) and returns elapsed
 * milliseconds; this ABI carries the same state behind an opaque engine
 * handle, takes plain pointers and sizes, returns an int status (0 = OK,
 * negative = error; never exit()) and reports milliseconds through an optional
 * out-parameter.  Layouts follow the reference:
 *   pos  float4 [n_atoms]: x, y, z, charge/sqrt(dielectric) (atom_class.h:31,
 *        read_prmtop.cpp:125)
 *   vel  float4 [n_atoms]: vx, vy, vz, mass with H masses reset to 12
 *        (atom_class.h:37, read_prmtop.cpp:141-146)
 *   force float4 [n_atoms]: fx, fy, fz, 0 (atom_class.h:33)
 * Units are the reference's: Angstrom, kcal/mol, amu, Amber time units
 * (dt = 0.002 ps * 20.455, config_class.cpp:123-124).
 *
 * Threading: one engine is driven by one host thread at a time; distinct
 * engines are independent.  All work of an engine runs on its own CUDA stream.
 */
#ifndef ISSPA_GB300_H
#define ISSPA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define ISSPA_OK 0
#define ISSPA_ERR_ARG (-1)          /* invalid argument / size */
#define ISSPA_ERR_IO (-2)           /* file could not be opened */
#define ISSPA_ERR_PARSE (-3)        /* malformed prmtop / isspatop / config / rst7 */
#define ISSPA_ERR_CUDA (-4)         /* CUDA runtime error */
#define ISSPA_ERR_NOMEM (-5)        /* allocation failed or over the engine's memory cap */
#define ISSPA_ERR_BOUNDS (-6)       /* a device-side bounds check tripped */
#define ISSPA_ERR_TIMEOUT (-7)      /* a bounded device wait gave up */
#define ISSPA_ERR_NONFINITE (-8)    /* a force or coordinate became NaN/Inf */
#define ISSPA_ERR_UNSUPPORTED (-9)  /* input outside what the engine supports */
#define ISSPA_ERR_STATE (-10)       /* call not valid in the engine's state */
#define ISSPA_ERR_OVERFLOW (-11)    /* a force exceeded the fixed-point range */
#define ISSPA_ERR_LIST_FULL (-12)   /* a neighbour-list row outgrew its capacity (cutoff mode) */

/* ---- system description (plain arrays) ---------------------------------- */
/* One simulation window: everything the reference's atom / bond / angle / dih
 * / isspa / us / config objects hold after setup (total_force_cuda.cpp:57-99).
 * All indices are 0-based.  The engine copies what it needs at creation. */
typedef struct isspa_system_desc {
    int n_atoms;
    const float *pos;            /* [n_atoms][4] */
    const float *vel;            /* [n_atoms][4]; .w = mass (H -> 12) */
    const float *raw_mass;       /* [n_atoms] prmtop masses (US mass fractions, us_class.cpp:147) */
    /* Lennard-Jones (read_prmtop.cpp:151-203, :353-384) */
    int n_lj_types;
    const int *lj_type;          /* [n_atoms] */
    const int *nb_parm_index;    /* [n_lj_types^2] index into lj_ab */
    const float *lj_ab;          /* [n_lj_types*(n_lj_types+1)/2][2]: A, B */
    /* exclusions (read_prmtop.cpp:167-186, :546-562): cumulative counts */
    int excl_len;
    const int *n_excl_cum;       /* [n_atoms] */
    const int *excl_list;        /* [excl_len] */
    /* bonded terms (read_prmtop.cpp:204-352, :386-545) */
    int n_bonds;
    const int *bond_atoms;       /* [n_bonds][3]: i, j, type */
    int n_bond_types;
    const float *bond_params;    /* [n_bond_types][2]: 2k, r0 */
    int n_angles;
    const int *angle_atoms;      /* [n_angles][4]: i, j, k, type */
    int n_angle_types;
    const float *angle_params;   /* [n_angle_types][2]: 2k, theta0 */
    int n_dihs;
    const int *dih_atoms;        /* [n_dihs][4]: i, j, +-k, +-l (sign flags as in Amber) */
    const int *dih_types;        /* [n_dihs] */
    int n_dih_types;
    const float *dih_params;     /* [n_dih_types][4]: periodicity, k, phase, 0 */
    const float *scaled14;       /* [n_dih_types][2]: SCEE, SCNB */
    /* IS-SPA solvent model (isspa_class.cpp:45-178) */
    const int *isspa_type;       /* [n_atoms] */
    int n_isspa_types;
    const float *rmax;           /* [n_isspa_types] */
    int n_g, n_e, n_f;           /* rows per type of ISSPA_DENSITIES / _EFIELD / _FORCES */
    const float *g_table;        /* [n_isspa_types][n_g] */
    const float *e_table;        /* [n_isspa_types][n_e] */
    const float *f_table;        /* [n_isspa_types][n_f] */
    float g_r0, g_dr, e_r0, e_dr, f_r0, f_dr;
    /* umbrella COM-distance restraint (us_class.cpp:13-158) */
    int us_on;
    int n_bias;
    const int *bias_list;        /* [n_bias][2]: atom, group (0/1) */
    float us_k, us_x0;
    /* run parameters (config_class.cpp:14-133) */
    int n_mc;
    float box;
    float kT;                    /* temperature * 0.00198717 */
    float dt;                    /* Amber time units */
    float pnu;                   /* Andersen collision probability per step */
    uint64_t seed;
} isspa_system_desc;

/* ---- engine options ------------------------------------------------------ */
typedef struct isspa_engine_options {
    int isspa_terms;     /* bit mask: 1 multipole, 2 tabulated LJ, 4 CDD; 0 => all (7);
                            ISSPA_TERMS_NONE => no IS-SPA pass at all */
    int nonbond_terms;   /* bit mask: 1 LJ, 2 Coulomb, 4 IS-SPA correction; 0 => all (7);
                            ISSPA_TERMS_NONE => no nonbond pass at all */
    int use_graph;       /* isspa_step captures the step in a CUDA graph (default 1) */
    int field_split;     /* atom-loop split per MC point in the field kernel; 0 => auto */
    int force_chunk;     /* MC points per force-kernel work item; 0 => auto */
    size_t mem_cap;      /* device bytes the engine may hold, including the temporary
                            buffers of the list queries; 0 => unlimited */
    int force_atoms_per_thread;  /* receiving atoms per IS-SPA force thread, 1 or 2; 0 => 1 */
    int force_tail_chunk;  /* MC points per force work item of the short items listed after
                              all force_chunk items (about two waves of them); 0 => none */
    int field_vote;      /* 1: the field pass walks its atoms in groups of four with one
                            warp vote on "any inside rmax" per group (same results);
                            0 => per-pair branches */
    int force_vote;      /* 1: the force pass (one atom per thread) takes its points in
                            groups of four with one warp vote per group (same results);
                            0 => per-pair branches */
    int integrator;      /* how isspa_step runs a step: 1 = bonded, umbrella and leapfrog
                            kernels (bonded, umbrella and nonbond on branches concurrent
                            with the IS-SPA pass);
                            2 = one fused cooperative kernel for bonded, umbrella and
                            leapfrog after the force passes; 3 = the whole step in one
                            cooperative kernel (field, nonbond, bonded | force | update,
                            with grid barriers; for latency-bound small systems; takes the
                            field split 4, and needs the tabulated LJ term, Philox points,
                            one receiving atom per force thread and at most 64 LJ types,
                            else 1).  Same results bit for bit for the same launch shapes;
                            0 => 1 until isspa_autotune times them all and keeps the fastest */
    int nonbond_chunk;   /* partners per nonbond work item (rounded up to a multiple of 128;
                            the results do not depend on it); 0 => auto */
    int field_tma;       /* 1: the field pass stages each round of 128 atoms with a 1-D bulk
                            copy (cp.async.bulk, the TMA engine) behind an mbarrier, double-
                            buffered (same results); 0 => coalesced loads by the threads */
    float nonbond_cutoff;  /* > 0: cutoff mode of the nonbond pass -- only pairs whose FP32
                              squared minimum-image distance is below cutoff^2 (A) count, with
                              LJ, Coulomb and the IS-SPA correction all truncated there (no
                              shift; energies likewise), found through a Verlet neighbour list
                              over per-window cell lists that the device rebuilds whenever an
                              atom has moved more than half the skin since the last build.
                              The forces do not depend on the skin or on when the list was
                              rebuilt.  Not available to isspa_adjoint_mean_force
                              (ISSPA_ERR_UNSUPPORTED) or to the single-kernel step (integrator 3
                              falls back to 1).  0 => every pair (the reference's behaviour: its
                              config `cutoff` reaches the nonbond kernel unused); < 0 or
                              non-finite => ISSPA_ERR_ARG */
    float nonbond_skin;    /* Verlet buffer of the neighbour list (A); 0 => 2 */
    int nonbond_list_max;  /* partners a neighbour-list row holds; 0 => 1.5 x the fullest row
                              of the starting configuration + 32 (at most the largest window).
                              A row that outgrows it reports ISSPA_ERR_LIST_FULL through
                              isspa_device_status (the forces of that step are incomplete) */
    int step_pdl;          /* 1: isspa_step launches the field, force and leapfrog kernels as
                              programmatic dependents of the kernel before each on the stream
                              (each waits for that kernel's completion before its first memory
                              access, so its launch overlaps the other's tail; same results);
                              2: ordinary launches; 0 => 2 until isspa_autotune times both and
                              keeps the faster.  The single-kernel step has no chain */
    int isspa_fused;       /* 1: the field and force passes run as one launch over the field
                              tiles: each block computes its points' fields, then those points'
                              forces on every atom of its window (for small windows; needs
                              Philox points, the tabulated LJ term and a field split of 4, 8 or
                              16, else the separate passes run).  Forces equal the separate
                              passes' up to FP32 summation order.  2: separate passes; 0 => 2
                              until isspa_autotune times both (windows of up to 512 atoms)
                              and keeps the faster */
    int force_overlap;     /* 1: in isspa_step the field blocks stamp their tiles when their
                              point records are written, and each force work item waits
                              (bounded; ISSPA_ERR_TIMEOUT from isspa_device_status if it gives
                              up) only for the tiles its points lie in, so with programmatic
                              launches the force pass starts in the field pass's last wave
                              (same results bit for bit; not with the fused launch or the
                              single-kernel step).  2: the force pass waits for the whole field
                              pass; 0 => 2 until isspa_autotune times both and keeps the faster */
} isspa_engine_options;

#define ISSPA_TERMS_NONE (-1)

typedef struct isspa_engine isspa_engine;
typedef struct isspa_host_system isspa_host_system;

const char *isspa_strerror(int status);
void isspa_default_options(isspa_engine_options *opt);
/* Number of CUDA devices visible to this process (0 when there is none). */
int isspa_device_count(int *count);

/* ---- input files (host side, no GPU needed) ------------------------------ */
/* Parsed `key = value` run configuration (config_class.cpp:14-133). */
typedef struct isspa_run_config {
    char prmtop[512], isspa_prmtop[512], input_coord[512], input_vel[512], us_cfg[512];
    char for_out[512], pos_out[512], vel_out[512], pos_rst_file[512], vel_rst_file[512];
    int n_mc, n_steps, delta_write, seed, us, vel_rst;
    int pnu_set;         /* 0 when the file gave no pnu (the reference leaves it uninitialised) */
    float temperature;   /* K, as given */
    float kT, dt, dt_ps, pnu, box, eps, cutoff;
} isspa_run_config;

/* Replaces config::initialize (config_class.cpp:14-133). */
int isspa_read_run_config(const char *path, isspa_run_config *out);
/* Reads prmtop (read_prmtop.cpp:10), isspatop (isspa_class.cpp:45), rst7
 * positions (atom_class.cpp:76-115), velocities (:117-156) or a seeded
 * Maxwell-Boltzmann draw (:53-64), and the US file (us_class.cpp:13-105).
 * Relative paths resolve against base_dir when it is non-NULL. */
int isspa_system_load(const isspa_run_config *cfg, const char *base_dir, isspa_host_system **out);
int isspa_read_prmtop(const char *path, float eps, isspa_host_system **out);
int isspa_read_isspatop(isspa_host_system *sys, const char *path);
/* Writes the IS-SPA sections of desc (types, rmax, density / field / force
 * tables with their radial grids) as an .isspatop file that
 * isspa_read_isspatop reads back exactly; replaces the table writer of
 * scripts/isspa_prmtop/write_isspa_prmtop.py:202-273, with ISSPA_FORCES in the
 * linear form the reader (isspa_class.cpp:155-170) uses. */
int isspa_write_isspatop(const isspa_system_desc *desc, const char *path, const char *title);
int isspa_read_rst7(isspa_host_system *sys, const char *path, int velocities);
int isspa_read_us_config(isspa_host_system *sys, const char *path, char *cv_file_out, size_t cv_len);
/* Points desc at the host system's arrays (valid until isspa_system_free). */
int isspa_system_describe(const isspa_host_system *sys, isspa_system_desc *desc);
int isspa_system_set_run(isspa_host_system *sys, int n_mc, float box, float kT, float dt,
                         float pnu, uint64_t seed);
void isspa_system_free(isspa_host_system *sys);

/* ---- engine lifetime ----------------------------------------------------- */
/* Creates an engine on the current CUDA device for n_windows independent
 * windows (umbrella windows or replicas) that share one force field: the same
 * LJ types/parameters, IS-SPA types/tables and n_mc.  n_windows == 1 is the
 * plain drop-in path (replaces the setup of total_force_cuda.cpp:77-99). */
int isspa_engine_create(const isspa_system_desc *windows, int n_windows,
                        const isspa_engine_options *opt, isspa_engine **out);
void isspa_engine_destroy(isspa_engine *e);
int isspa_engine_info(const isspa_engine *e, int *n_windows, int *n_atoms_total,
                      long long *n_points_total);
/* Launch shapes the engine chose (or was given) for its work lists:
 * shape[0] field atom-loop split, [1] field tiles, [2] force points per work
 * item, [3] force work items, [4] nonbond work items, [5] nonbond partners per
 * item, [6] SM count used for the choice, [7] receiving atoms per force
 * thread, [8] points per force work item of the short items listed last (0:
 * none), [9] 1 when the field pass walks its atoms in warp-voted groups,
 * [10] 1 when the force pass takes its points in warp-voted groups, [11] the
 * step integrator (1 separate kernels, 2 fused, 3 single-kernel step; see isspa_engine_options),
 * [12] 1 when the field pass stages its atoms by bulk copies (TMA), [13] in
 * cutoff mode the partners a neighbour-list row holds (0 otherwise), [14] in
 * cutoff mode the cells of all windows' cell grids (0 otherwise), [15] 1 when
 * isspa_step launches its kernel chain as programmatic dependents, [16] 1 when
 * the field and force passes run as one fused launch, [17] 1 when the step's
 * force items start on stamped field tiles (force_overlap). */
#define ISSPA_SHAPE_COUNT 18
int isspa_engine_shapes(const isspa_engine *e, int shape[ISSPA_SHAPE_COUNT]);
/* Autotuner: times every field-pass atom split (per-pair and warp-voted
 * loops, atoms staged by loads or by bulk copies) and, for 1 and 2 receiving
 * atoms per force thread, a set of force-pass chunk lengths (those filling
 * 1..12 whole waves of resident blocks, and powers of two; and long chunks
 * followed by about two waves of short ones; then the voted force loop on the
 * chosen list) on this engine's own
 * workload with CUDA events (reps launches each), keeps the fastest of each
 * and reports the result as isspa_engine_shapes does.  When the options leave
 * the integrator, step_pdl, isspa_fused or force_overlap open (0), it then
 * times single-step graph replays of the open choices (separate kernels, fused
 * integrator, single-kernel step; with and without programmatic launches;
 * the fused field + force launch or the separate passes, with and without
 * force_overlap) and keeps the fastest (the nonbond
 * partners per item are timed too); positions,
 * velocities and the step counter are restored.  Clears the force
 * accumulator; invalidates captured graphs. */
int isspa_autotune(isspa_engine *e, int reps, int shape[ISSPA_SHAPE_COUNT]);

/* ---- per-step force calls (reference names and order) -------------------- */
/* Each call adds its forces into the engine's force accumulator, exactly as the
 * reference kernels add into for_d.  With ms_out != NULL the call is timed
 * with CUDA events and synchronises (like the reference wrappers); with NULL it
 * is only enqueued on the engine stream. */
int isspa_zero_forces(isspa_engine *e);                   /* cudaMemset(for_d), total_force_cuda.cpp:109 */
int bond_force_cuda(isspa_engine *e, float *ms_out);      /* bond_force_cuda.cu:58-79 */
int angle_force_cuda(isspa_engine *e, float *ms_out);     /* angle_force_cuda.cu:69-86 */
int dih_force_cuda(isspa_engine *e, float *ms_out);       /* dih_force_cuda.cu:140-157 */
int isspa_force_cuda(isspa_engine *e, float *ms_out);     /* isspa_force_cuda.cu:331-360 */
int nonbond_force_cuda(isspa_engine *e, float *ms_out);   /* nonbond_force_cuda.cu:178-194 */
int us_force_cuda(isspa_engine *e, float *ms_out);        /* us_force_cuda.cu:50-69 */
int leapfrog_cuda(isspa_engine *e, float *ms_out);        /* leapfrog_cuda.cu:73-86; advances the step counter */

/* Runs nsteps complete MD steps (zero, bonded, IS-SPA, nonbond, US, leapfrog)
 * in the reference order, replayed from a captured CUDA graph. */
int isspa_step(isspa_engine *e, int nsteps);
/* Runs nsteps steps and returns their device time (CUDA events on the engine
 * stream).  flush_bytes > 0 writes that many bytes of scratch between steps
 * (outside the timed intervals) to evict L2. */
int isspa_time_steps(isspa_engine *e, int nsteps, size_t flush_bytes, double *ms_total);
/* As isspa_time_steps, also timing every kernel of the step with CUDA events
 * recorded on the stream each kernel runs on, inside the replayed graph.
 * ms_kernels[ISSPA_K_COUNT] receives the summed milliseconds per kernel and
 * launches[ISSPA_K_COUNT] the number of launches of each. */
enum { ISSPA_K_FIELD = 0, ISSPA_K_FORCE, ISSPA_K_NONBOND, ISSPA_K_BONDED, ISSPA_K_UMBRELLA,
       ISSPA_K_LEAPFROG, ISSPA_K_INTEGRATOR, ISSPA_K_STEP, ISSPA_K_COUNT };
int isspa_time_steps_detailed(isspa_engine *e, int nsteps, size_t flush_bytes, double *ms_total,
                              double *ms_kernels, int *launches);
/* Page-locked host buffers, mapped into the device address space
 * (cudaHostAlloc, portable and mapped).  The library keeps a registry of the
 * live ones: isspa_step_host reads and writes buffers inside them from the GPU
 * directly.  Release them with isspa_host_free only (never cudaFreeHost), so
 * that the registry never holds a freed range. */
int isspa_host_alloc(size_t bytes, void **out);
void isspa_host_free(void *p);
int isspa_synchronize(isspa_engine *e);
/* Sticky device status word (0 if nothing tripped); clears it when reset != 0. */
int isspa_device_status(isspa_engine *e, int reset);
/* Cutoff mode (no counterpart on the reference's live path; its dead
 * neighborlist_cuda.cu:11-137 / cell_list_cuda.cu:13-35 are the closest):
 * how many times the neighbour list has been built since the engine was made,
 * and the fullest row of the last build (partners within cutoff + skin).
 * Synchronises the engine stream.  ISSPA_ERR_STATE without a cutoff. */
int isspa_nonbond_list_stats(isspa_engine *e, int *builds, int *fullest_row);
/* Failure-detection testing (no counterpart in the reference): leaves the
 * fused integrator's grid barrier as if a block had been lost mid-count, so the
 * next fused step's bounded waits run out; that step integrates nothing and
 * reports ISSPA_ERR_TIMEOUT through isspa_device_status, whose reset also
 * restores the barrier.  No kernel faults and the context stays usable. */
int isspa_debug_stall_barrier(isspa_engine *e);

/* ---- state transfer (host <-> device, synchronous) ----------------------- */
int isspa_set_positions(isspa_engine *e, const float *pos4, int n_atoms_total);
int isspa_get_positions(isspa_engine *e, float *pos4, int n_atoms_total);
int isspa_set_velocities(isspa_engine *e, const float *vel4, int n_atoms_total);
int isspa_get_velocities(isspa_engine *e, float *vel4, int n_atoms_total);
/* Current contents of the force accumulator (float4, .w = 0). */
int isspa_get_forces(isspa_engine *e, float *f4, int n_atoms_total);
int isspa_set_step(isspa_engine *e, uint32_t step);
int isspa_get_step(isspa_engine *e, uint32_t *step);
/* Umbrella COM of both groups per window (double [n_windows][2][3]) and the
 * collective variable |COM0 - COM1| (double [n_windows]) of the last us call. */
int isspa_get_us_com(isspa_engine *e, double *com, double *cv);

/* One MD step with host buffers: upload pos/vel, run one full step, download
 * pos/vel/force (float [n_atoms_total][4] each; any may be NULL).  This is
 * the call a host-side driver makes per step.  When every non-NULL buffer is a
 * 16-byte aligned range inside isspa_host_alloc memory, two small kernels move
 * the state over the host link around the step, launched with it as one graph
 * per set of buffers (the last four sets kept); otherwise one copy per buffer.
 * Same results either way. */
int isspa_step_host(isspa_engine *e, const float *pos_in, const float *vel_in, float *pos_out,
                    float *vel_out, float *force_out);

/* ---- IS-SPA point-set access (parity with other implementations) -------- */
/* Injects MC point positions (float [n_points_total][3]); subsequent
 * isspa_force_cuda calls use them instead of generating Philox points, until
 * isspa_clear_mc_points. */
int isspa_set_mc_points(isspa_engine *e, const float *xyz, long long n_points_total);
int isspa_clear_mc_points(isspa_engine *e);
/* Per-point results of the last field pass: positions [P][3], density
 * product w [P], in-range count n [P], mean field E [P][3], far field E0 [P][3]. */
int isspa_get_point_fields(isspa_engine *e, float *xyz, float *w, int *n, float *efield,
                           float *e0field, long long n_points_total);

/* ---- force-field parameters and their gradient --------------------------- */
/* Replaces the engine's tables (host arrays in the layouts of
 * isspa_system_desc; NULL keeps a table): ISSPA_DENSITIES, ISSPA_EFIELD,
 * ISSPA_FORCES, and the packed LJ A/B coefficients.  Shapes are unchanged. */
int isspa_set_tables(isspa_engine *e, const float *g_table, const float *e_table, const float *f_table,
                     const float *lj_ab);
/* Mean COM-axis force of every restrained window and its gradient with
 * respect to the force field (no counterpart in the reference, which has no
 * derivatives).  For frame f the engine's positions are frames[f] ([Ntot][4];
 * NULL = the current positions) and the MC points are regenerated from the
 * Philox counters of steps[f] (no point storage).  With c_i = +n/2 on restraint
 * group 0 and -n/2 on group 1 (n the unit vector between the group centres of
 * mass, us_force_cuda.cu:30-34), J_w = mean_f sum_i c_i . F_i, F_i the total
 * non-restraint force (bonded, IS-SPA, nonbond).  Outputs per window, FP64:
 *   J [n_windows], dJ_df [n_windows][n_isspa_types*n_f] (ISSPA_FORCES entries),
 *   dJ_dg [n_windows][n_isspa_types*n_g] (ISSPA_DENSITIES entries),
 *   dJ_dA, dJ_dB [n_windows][n_lj_types*(n_lj_types+1)/2] (packed LJ A, B).
 * Windows without a restraint get zeros.  The engine's positions and step
 * counter are restored; the force accumulator is cleared.  Any output may be
 * NULL. */
int isspa_adjoint_mean_force(isspa_engine *e, int n_frames, const float *frames, const uint32_t *steps,
                             double *J, double *dJ_df, double *dJ_dg, double *dJ_dA, double *dJ_dB);

/* ---- energies and virial (no counterpart in the reference, which reports
 * none) ------------------------------------------------------------------- */
/* Components of isspa_energies, kcal/mol, per window:
 *   KIN_BEFORE  sum m v^2/2 with the stored half-step velocities v(t-dt/2);
 *   KIN_AFTER   the same with v(t+dt/2) = v(t-dt/2) + F(t) dt/m, the
 *               thermostat-free leapfrog kick (leapfrog_cuda.cu:57-60);
 *               the kinetic energy at t is their mean;
 *   BOND        sum k (r - r0)^2           (bond_force_cuda.cu:36-50, 2k stored)
 *   ANGLE       sum k (theta - theta0)^2   (angle_force_cuda.cu:19-52)
 *   DIHEDRAL    sum V (1 + cos(n phi - phase))   (dih_force_cuda.cu:86-135)
 *   LJ14, COUL14  scaled 1-4 terms          (dih_force_cuda.cu:60-82)
 *   LJ, COUL    A/r^12 - B/r^6 and q q / r over non-excluded pairs
 *               (nonbond_force_cuda.cu:131-136)
 *   CORR        the potential of the IS-SPA dielectric correction
 *               (nonbond_force_cuda.cu:141-147), zero at infinity; it is the
 *               pair potential of the force only when every IS-SPA type has
 *               the same rmax (each ordered pair uses rmax of the partner)
 *   UMBRELLA    k/2 (|COM0 - COM1| - x0)^2  (us_force_cuda.cu:14-48)
 *   VIRIAL      sum r . F over the conservative terms above (pair, bonded
 *               and restraint forces); the IS-SPA mean-field force has no
 *               potential and is in neither the energy nor the virial.
 * Each term follows the engine's term options.  Pair energies are evaluated
 * in FP32 like the forces; every reduction is in FP64. */
enum { ISSPA_E_KIN_BEFORE = 0, ISSPA_E_KIN_AFTER, ISSPA_E_BOND, ISSPA_E_ANGLE, ISSPA_E_DIHEDRAL,
       ISSPA_E_LJ14, ISSPA_E_COUL14, ISSPA_E_LJ, ISSPA_E_COUL, ISSPA_E_CORR, ISSPA_E_UMBRELLA,
       ISSPA_E_VIRIAL, ISSPA_E_COUNT };
/* Energies of the engine's current state: computes the forces of the current
 * step (every enabled term, MC points of the current step counter) into the
 * accumulator, reduces the components above into out[n_windows][ISSPA_E_COUNT]
 * and clears the accumulator again.  Positions, velocities and the step
 * counter are not changed, so isspa_step continues the same trajectory. */
int isspa_energies(isspa_engine *e, double *out);

/* ---- neighbour and cell lists (neighborlist_cuda.cu, cell_list_cuda.cu) -- */
/* All-pairs neighbour list of window 0 with r^2 < rnn^2, exclusions as the
 * nonbond kernel; rows sorted ascending.  rows [n_atoms][max_per_atom], counts
 * [n_atoms] (counts may exceed max_per_atom: rows then hold the first
 * max_per_atom partners in ascending order). */
int isspa_neighbor_list(isspa_engine *e, float rnn, int max_per_atom, int *rows, int *counts);
/* Cell index of every atom of window 0 (cell_list_cuda.cu:27-29). */
int isspa_cell_list(isspa_engine *e, float rc, const int ncell[3], int *cell_of_atom);

/* Device FP32 throughput probe: runs a dependent-chain FMA kernel over the whole
 * GPU and returns the measured TFLOP/s (FMA = 2 flops). */
int isspa_measure_fp32_peak(double *tflops);

/* ---- IS-SPA force without any allocation ---------------------------------
 * No counterpart in the reference.  For callers that must not call cudaMalloc
 * (or any allocating routine): code running inside another framework's memory
 * pool, a host process whose device memory is budgeted up front, or a real-time
 * loop that may not take the allocator's locks.  All arrays below are DEVICE
 * pointers owned by the caller; the work lists, per-point field records, packed
 * tables, force accumulator and status word live in one static device buffer
 * of ISSPA_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds
 * until the process exits.  The buffer needs 80 bytes per MC point, 32 per atom
 * and the work lists (16 bytes per 32-128 points and per force work item);
 * systems that do not fit are rejected with ISSPA_ERR_UNSUPPORTED before
 * anything is enqueued (roughly 200 k MC points, e.g. 3900 atoms at nMC 50).
 * The first call on a device looks up that buffer's device address; make that
 * first call before any stream capture.  Calls share the buffer, so calls
 * that overlap on the GPU (different streams) race and must be ordered by the
 * caller.  Computes the same IS-SPA force as isspa_force_cuda for one window and
 * writes it to force_out ([n_atoms][4], .w = 0), on `stream` (a cudaStream_t;
 * NULL = legacy default stream), without synchronising and without any
 * host-to-device copy.  The return value reports argument and launch errors;
 * what the kernels find (a force beyond the fixed-point range, a non-finite
 * force, an IS-SPA type outside [0, n_isspa_types), which is then read as type
 * 0) is written as ISSPA_NOALLOC_STATUS_* bits to *status_out when that pointer
 * is given, ordered after force_out on the same stream. */
#define ISSPA_NOALLOC_SCRATCH_BYTES (16u << 20)
#define ISSPA_NOALLOC_STATUS_OVERFLOW 1   /* a force beyond the fixed-point accumulator's range */
#define ISSPA_NOALLOC_STATUS_NONFINITE 2  /* a non-finite force */
#define ISSPA_NOALLOC_STATUS_BOUNDS 4     /* an index out of range (IS-SPA type) */
typedef struct isspa_noalloc_inputs {
    int n_atoms, n_mc, n_isspa_types;
    const float *pos;         /* [n_atoms][4]: x, y, z, charge/sqrt(eps) */
    const int *isspa_type;    /* [n_atoms] */
    const float *rmax;        /* [n_isspa_types] */
    int n_g, n_e, n_f;
    const float *g_table, *e_table, *f_table; /* [n_isspa_types][n_g | n_e | n_f] */
    float g_r0, g_dr, e_r0, e_dr, f_r0, f_dr;
    float box;
    uint64_t seed;
    uint32_t step;            /* Philox step key of the MC points */
    int terms;                /* 1 multipole, 2 tabulated LJ, 4 CDD, any sum of them; 0 => all;
                                 other values => ISSPA_ERR_ARG */
    int *status_out;          /* optional device-accessible int (device or mapped host memory):
                                 receives this call's ISSPA_NOALLOC_STATUS_* bits, 0 = clean */
} isspa_noalloc_inputs;
int isspa_force_noalloc(const isspa_noalloc_inputs *in, float *force_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ISSPA_GB300_H */
