// kernels.h -- argument blocks and launch wrappers of the device kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"

namespace isspa {

// ---- IS-SPA field pass (one thread-column per MC point) ------------------
struct FieldArgs {
    const float4 *pos;     // [Ntot] x, y, z, q
    const int2 *atype;     // [Ntot] lj type, isspa type
    const WinDev *win;
    const int4 *tiles;     // [n_tiles] window, first point (global), n points, 0
    int n_tiles;
    const float4 *gtab;    // [n_itypes * n_gbins] g_b, g_b+1, e_b, e_b+1
    const float *rmax;     // [n_itypes]
    int n_gbins;           // nG - 1
    float g_r0, g_dr, g_inv, e_r0, e_dr, e_inv;
    float e0;
    int n_mc;
    uint32_t seed_lo, seed_hi;
    const uint32_t *step_ptr;  // device step counter
    const float *pts_in;   // injected points [P][3] (global order) or nullptr
    PointsDev out;
    float4 *raw_e;         // optional: E, w
    float4 *raw_e0;        // optional: E0, n
    int terms;             // IS-SPA force terms: 1 multipole, 2 tabulated LJ, 4 CDD
    int *status;
    int vote;              // 1: atom loop in warp-voted groups of four (same results)
    int tma;               // 1: atom rounds staged by 1-D bulk copies (TMA) behind mbarriers (same results)
    // overlap with the force pass: each block stamps tile_flag[tile] with
    // *ov_epoch + 1 once its records are written (nullptr: no stamps)
    unsigned int *tile_flag;
    const unsigned int *ov_epoch;
};

// ---- IS-SPA force pass (one thread per receiving atom) -------------------
struct ForceArgs {
    const float4 *pos;
    const int2 *atype;
    const WinDev *win;
    const int4 *items;     // window, first atom (global), n atoms, chunk index
    const int2 *chunks;    // [chunk index]: first point (global), n points
    int n_items;
    PointsDev pts;
    const float2 *ftab;    // [n_itypes * n_f] packed (f_k, f_k+1), flat semantics
    const float *rmax;
    const float *vtot;
    int n_f;
    float f_r0, f_dr, f_inv;
    int terms;             // 1 multipole, 2 tabulated LJ, 4 CDD
    int atoms_per_thread;  // 1 (128-thread blocks) or 2 (64-thread blocks)
    int vote;              // 1: points in warp-voted groups of four (same results)
    unsigned long long *facc;  // [Ntot][3]
    int *status;
    // overlap with the field pass (overlap = 1): instead of waiting for the
    // whole field kernel, an item waits (bounded) for the stamps of the field
    // tiles its chunk covers (tile_base[window] + point / tile_pts); the
    // update kernel advances *ov_epoch with the step counter
    int overlap;
    const unsigned int *tile_flag;
    unsigned int *ov_epoch;
    const int *tile_base;
    int tile_pts;
};

// ---- all-pairs nonbond --------------------------------------------------
struct NonbondArgs {
    const float4 *pos;
    const int2 *atype;
    const int *atom_win;       // [Ntot]
    const WinDev *win;
    const int4 *items;         // window, first i (global), n i, first j (global)
    const int *items_nj;       // [n_items]
    int n_items;
    const float2 *ljab;        // [n_lj_types^2] A, B (expanded from nb_parm_index)
    int n_lj_types;
    const float *rmax;
    const int *excl_start;     // [Ntot+1] CSR of symmetric exclusions (global, sorted)
    const int *excl;
    int terms;                 // 1 LJ, 2 Coulomb, 4 IS-SPA correction
    float cut2;                // pair energies: squared cutoff (+inf: every pair)
    unsigned long long *facc;
    int *status;
};

// ---- cutoff nonbond: Verlet neighbour list over cell lists ---------------
struct NbListArgs {
    const float4 *pos;
    const int2 *atype;
    const int *atom_win;
    const WinDev *win;
    const int4 *wcell;         // per window: first cell, cells per edge (1: one cell), bits of nc / box, -
    int n_atoms;               // all windows
    int n_cells;               // all windows
    float4 *ref;               // [Ntot] positions at the last build (NaN before the first)
    int *flag;                 // 1: rebuild this step
    int *stats;                // builds so far, fullest row of the last build
    int *cell_of, *cell_count, *cell_start, *cell_cursor, *cell_atoms;
    int *rows;                 // [Ntot][row_cap] partner | excluded << 31 (nullptr: counts only)
    int *row_n;                // [Ntot] partners found (may exceed row_cap)
    int row_cap;
    float half_skin2;          // (skin / 2)^2
    float list2;               // (cutoff + skin)^2
    float cut2;                // cutoff^2
    const int *excl_start, *excl;
    const float2 *ljab;
    int n_lj_types;
    const float *rmax;
    int terms;                 // 1 LJ, 2 Coulomb, 4 IS-SPA correction
    unsigned long long *facc;
    int *status;
};

// ---- bonded + umbrella ----------------------------------------------------
struct BondedArgs {
    const float4 *pos;
    const int *atom_win;
    const WinDev *win;
    const int4 *bonds;         // i, j, type, -
    int n_bonds;
    const float2 *bond_par;    // 2k, r0
    const int4 *angles;        // i, j, k, type
    int n_angles;
    const float2 *angle_par;
    const float4 *angle_cs;    // cos theta0 (hi, lo), sin theta0 (hi, lo): double-float per angle type
    const int4 *dihs;          // i, j, +-k, +-l
    const int *dih_type;
    int n_dihs;
    const float4 *dih_par;     // n, k, phase, -
    const float2 *sc14;        // scee, scnb
    const float2 *ljab;
    const int2 *atype;
    int n_lj_types;
    int do_bonds, do_angles, do_dihs;
    unsigned long long *facc;
    int *status;
};

struct UmbrellaArgs {
    const float4 *pos;
    const WinDev *win;
    const int *us_windows;     // windows with a restraint
    int n_us_windows;
    const int2 *bias;          // global atom, group
    const float *mfrac;        // mass fraction within its group
    double *com;               // [n_windows][2][3]
    double *cv;                // [n_windows]
    unsigned long long *facc;
    int *status;
};

struct LeapfrogArgs {
    float4 *pos;
    float4 *vel;
    float4 *force_out;         // converted forces of this step
    unsigned long long *facc;  // read and cleared
    const int *atom_win;
    const WinDev *win;
    int n_atoms;
    uint32_t seed_lo, seed_hi;
    uint32_t *step_ptr;        // advanced by the last block to finish
    unsigned int *done_ptr;    // block-completion counter (self-resetting)
    int *status;
    unsigned int *ov_epoch;    // advanced with the step counter (the field-tile stamps' base)
};

// Fused integrator: the bonded terms, the umbrella restraint and leapfrog of a
// step in one cooperative launch (a grid barrier between the force terms and
// the update).
struct IntegratorArgs {
    BondedArgs bonded;
    UmbrellaArgs us;
    LeapfrogArgs lf;
    const int *bias_start;     // [Ntot+1]: atom i's bias entries are bias_by_atom[bias_start[i]..bias_start[i+1])
    const int *bias_by_atom;   // global bias entry indices, grouped by atom
    double2 *usf;              // [n_windows][2]: COM axis r and (|r| - x0)/|r| of the step
    unsigned int *bar;         // grid barrier: arrival count, generation (zero at rest)
};

// The whole MD step of an engine in one cooperative launch (see step_kernel).
struct StepArgs {
    FieldArgs field;
    ForceArgs force;
    NonbondArgs nonbond;
    IntegratorArgs integ;
};

struct ListArgs {
    const float4 *pos;
    const int *excl_start;
    const int *excl;
    int atom_off, n_atoms;
    float box, hbox, rnn2;
    int max_per_atom;
    int *rows;                 // [n][max_per_atom]
    int *counts;
};

// ---- adjoint of the mean COM-axis force ------------------------------------
struct AdjointArgs {
    const float4 *pos;
    const int2 *atype;
    const WinDev *win;
    const int *atom_win;
    long long n_points;
    const int *point_win;      // [Ptot]
    const float4 *raw_e;       // field pass: E, w
    const float4 *raw_e0;      // field pass: E0, n
    const float4 *q0;          // point positions
    const int *adj_off;        // [n_windows+1] ranges of adj_atoms per window
    const int *adj_atoms;      // atoms with a nonzero weight
    int n_adj;
    const double *cvec;        // [Ntot][3] weights c_i
    const float *rmax, *vtot;
    float f_r0, f_dr, f_inv;
    int n_f;
    const float2 *ftab;
    long long n_ftab;          // n_itypes * n_f
    double *dJ_df;             // [n_windows][n_ftab]
    double *lam;               // [Ptot] dJ/ds_p
    const float *g_table;      // flat ISSPA_DENSITIES
    int n_g;
    float g_r0, g_dr, g_inv;
    long long n_gtab;          // n_itypes * n_g
    double *dJ_dg;             // [n_windows][n_gtab]
    int n_mc;
    const int *excl_start, *excl;
    const int *nbp;            // [n_lj_types^2] packed LJ index
    int n_lj_types;
    int n_ljtab;               // n_lj_types (n_lj_types + 1) / 2
    double *dJ_dA, *dJ_dB;     // [n_windows][n_ljtab]
    const int4 *dihs;
    const int *dih_type;
    int n_dihs;
    const float2 *sc14;
};

// ---- energies and virial (FP64 reductions) ----------------------------------
// Component slots, identical to the ISSPA_E_* enum of the public header.
enum EnergySlot {
    kEKinBefore = 0, kEKinAfter, kEBond, kEAngle, kEDihedral, kELj14, kECoul14, kELj, kECoul, kECorr,
    kEUmbrella, kEVirial, kECount
};
struct StateEnergyArgs {
    const float4 *vel;                 // v(t - dt/2), mass in .w
    const unsigned long long *facc;    // F(t), fixed point
    const int *atom_win;
    const WinDev *win;
    int n_atoms;
    const int *us_windows;             // restrained windows and their CV
    int n_us_windows;
    const double *cv;
};
void launch_nonbond_energy(const NonbondArgs &a, double *energy, cudaStream_t s);
void launch_bonded_energy(const BondedArgs &a, double *energy, cudaStream_t s);
void launch_state_energy(const StateEnergyArgs &a, double *energy, cudaStream_t s);

// ---- the step's main chain: field -> force -> leapfrog ---------------------
// While a PdlScope lives on a thread, the chain's kernels (each opens with
// pdl_wait) are launched from that thread as programmatic dependents of the
// kernel before them on the stream: a kernel's launch and block scheduling
// overlap the tail of the one it depends on.  Every other kernel, and the
// chain outside such a scope, launches as an ordinary kernel.
bool chain_pdl();
class PdlScope {
  public:
    explicit PdlScope(bool on);
    ~PdlScope();
    PdlScope(const PdlScope &) = delete;
    PdlScope &operator=(const PdlScope &) = delete;

  private:
    bool prev_;
};
#ifdef __CUDACC__
template <class... P, class... A>
inline void launch_chain(void (*k)(P...), unsigned grid, unsigned block, cudaStream_t s, const A &...args) {
    if (!chain_pdl()) {
        k<<<grid, block, 0, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);  // a failure is the thread's last error
}
#endif

void launch_adjoint(const AdjointArgs &a, cudaStream_t s);
void launch_field(const FieldArgs &a, int split, bool raw, cudaStream_t s);
void launch_force(const ForceArgs &a, cudaStream_t s);
// Field and force passes as one launch over the field tiles (split 4, 8 or
// 16, Philox points, tabulated LJ term on): each tile's points act on every
// atom of its window right after their fields are known.
bool field_force_fusable(int split);
void launch_field_force(const FieldArgs &f, const ForceArgs &g, int split, cudaStream_t s);
void launch_nonbond(const NonbondArgs &a, cudaStream_t s);
// Cutoff mode: displacement check and (when it trips) the list rebuild; then the pairs.
void launch_nblist_build(const NbListArgs &a, cudaStream_t s);
void launch_nblist_pairs(const NbListArgs &a, cudaStream_t s);
void launch_bonded(const BondedArgs &a, cudaStream_t s);
void launch_umbrella(const UmbrellaArgs &a, cudaStream_t s);
void launch_leapfrog(const LeapfrogArgs &a, cudaStream_t s);
// Cooperative launch of the fused integrator on `grid` blocks (at most
// integrator_max_blocks()); returns the launch's error code.
cudaError_t launch_integrator(const IntegratorArgs &a, int grid, cudaStream_t s);
int integrator_max_blocks();
int integrator_block_threads();
// Cooperative launch of the single-kernel step (field split 4, one receiving
// atom per force thread, LJ table in shared memory, tabulated LJ term on).
cudaError_t launch_step(const StepArgs &a, int grid, cudaStream_t s);
int step_max_blocks(int n_lj_types);
int step_threads();
void launch_neighbor_list(const ListArgs &a, cudaStream_t s);
// Up to three float4 arrays of n elements copied element-wise (a null source
// skips its pair): state moved between the engine's device arrays and
// page-locked host buffers that the GPU reads and writes directly.
struct Copy3Args {
    const float4 *src[3];
    float4 *dst[3];
    int n;
};
void launch_copy3(const Copy3Args &a, cudaStream_t s);
void launch_cell_index(const float4 *pos, int atom_off, int n, float rc, int3 ncell, int *cell,
                       cudaStream_t s);
double measure_fp32_peak_tflops();
int field_block_threads();
int force_block_threads();
int nonbond_block_threads();
// launch-shape helpers for the work-list builder
int field_points_per_block(int split);
int field_blocks_per_sm(int split);
int force_blocks_per_sm(int atoms_per_thread);
int nonbond_blocks_per_sm(int n_lj_types);

}  // namespace isspa
