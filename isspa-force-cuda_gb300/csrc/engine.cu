// engine.cu -- the engine object behind the C ABI: device memory layout,
// work lists, the per-step call sequence and its CUDA-graph capture.
//
// Device layout (one engine = one batch of windows sharing a force field):
//   pos, vel, force_out   float4 [Ntot]        (reference atom_class.h:31-38)
//   facc                  int64  [Ntot][3]     fixed-point force accumulator
//   atype                 int2   [Ntot]        LJ type, IS-SPA type
//   atom_win              int    [Ntot]
//   points (SoA float4)   [Ptot] x5            per-point field-pass results (q0..q4)
//   tables                g/E packed float4, force packed float2, LJ A/B float2
// Windows are concatenated; every work list is built once at creation.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "host_system.h"
#include "isspa_gb300.h"
#include "kernels.h"

using namespace isspa;

namespace {

constexpr int kStepsPerGraph = 8;

// Page-locked buffers handed out by isspa_host_alloc and not yet freed:
// host start -> (bytes, device address of the start).
std::mutex g_host_mu;
std::map<uintptr_t, std::pair<size_t, uintptr_t>> g_host_bufs;

// Device address of the host range [p, p + bytes) when it is 16-byte aligned
// and lies inside one live isspa_host_alloc buffer; nullptr otherwise (any
// other memory is only ever reached through cudaMemcpyAsync).
void *host_mapped(const void *p, size_t bytes) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    if (!p || a % 16) return nullptr;
    std::lock_guard<std::mutex> lock(g_host_mu);
    auto it = g_host_bufs.upper_bound(a);
    if (it == g_host_bufs.begin()) return nullptr;
    --it;
    if (a - it->first > it->second.first || bytes > it->second.first - (a - it->first)) return nullptr;
    return reinterpret_cast<void *>(it->second.second + (a - it->first));
}

struct Fail {
    int code;
};

inline void ck(cudaError_t e) {
    if (e != cudaSuccess) throw Fail{ISSPA_ERR_CUDA};
}

}  // namespace

struct isspa_engine {
    int device = 0;
    cudaStream_t stream = nullptr, side = nullptr, side2 = nullptr, side3 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr, ev_join3 = nullptr, ev_a = nullptr,
                ev_b = nullptr;
    isspa_engine_options opt{};
    int n_windows = 0, n_atoms = 0, n_mc = 0;
    long long n_points = 0;
    std::vector<WinDev> win_h;
    std::vector<void *> allocs;
    size_t allocated = 0;

    // device state
    float4 *pos = nullptr, *vel = nullptr, *force_out = nullptr;
    unsigned long long *facc = nullptr;
    int2 *atype = nullptr;
    int *atom_win = nullptr;
    WinDev *win = nullptr;
    float4 *gtab = nullptr;
    float2 *ftab = nullptr, *ljab = nullptr;
    float *rmax = nullptr, *vtot = nullptr;
    int *excl_start = nullptr, *excl = nullptr;
    int4 *field_tiles = nullptr;
    int n_field_tiles = 0, field_split = 4;
    int4 *force_items = nullptr;
    int2 *force_chunks = nullptr;
    int n_force_items = 0, force_chunk = 0;
    int force_tail = 0;  // chunk length of the short items listed last (0: none)
    int field_vote = 0;  // field pass in warp-voted groups of four atoms
    int field_tma = 0;   // field pass stages its atom rounds by 1-D bulk copies (TMA)
    int step_pdl = 0;    // step chain launched as programmatic dependents (1) or not (0)
    int isspa_fused = 0;  // field and force passes as one launch (1) when fused_ok()
    int force_overlap = 0;  // force items start on stamped field tiles (1) when overlap_ok()
    unsigned int *tile_flag = nullptr;  // per field tile: the stamp of the pass that wrote its records
    size_t tile_flag_cap = 0;
    int *tile_base = nullptr;           // per window: its first field tile
    unsigned int *ov_epoch = nullptr;   // stamp of the current pass - 1 (advanced with the step counter)
    int force_vote = 0;  // force pass in warp-voted groups of four points (1 atom per thread)
    int force_apt = 1;  // receiving atoms per force-kernel thread (1 or 2)
    // step integrator: 1 = bonded, umbrella and leapfrog kernels (bonded and
    // umbrella on the forked branch), 2 = one fused cooperative kernel
    int integrator = 1;
    int integ_grid = 0;
    int *bias_start = nullptr, *bias_by_atom = nullptr;
    double2 *usf = nullptr;
    unsigned int *bar = nullptr;
    int4 *nb_items = nullptr;
    int *nb_nj = nullptr;
    int n_nb_items = 0, nb_chunk = 0, n_sms = 0;
    // cutoff mode of the nonbond pass (nonbond_cutoff > 0): Verlet list over cell lists
    bool cutoff = false;
    float nb_cut2 = 0.f, nb_list2 = 0.f, nb_half_skin2 = 0.f;
    int4 *nbl_wcell = nullptr;
    float4 *nbl_ref = nullptr;
    int *nbl_flag = nullptr, *nbl_stats = nullptr;
    int *nbl_cell_of = nullptr, *nbl_cell_count = nullptr, *nbl_cell_start = nullptr, *nbl_cell_cursor = nullptr,
        *nbl_cell_atoms = nullptr, *nbl_rows = nullptr, *nbl_row_n = nullptr;
    int nbl_cells = 0, nbl_row_cap = 0;
    int4 *bonds = nullptr, *angles = nullptr, *dihs = nullptr;
    float2 *bond_par = nullptr, *angle_par = nullptr, *sc14 = nullptr;
    float4 *angle_cs = nullptr;
    float4 *dih_par = nullptr;
    int *dih_type = nullptr;
    int n_bonds = 0, n_angles = 0, n_dihs = 0;
    int *us_windows = nullptr;
    int n_us = 0;
    int2 *bias = nullptr;
    float *mfrac = nullptr;
    std::vector<int2> bias_h;
    std::vector<float> mfrac_h, lj_ab_h, g_raw_h, e_raw_h, f_raw_h;
    std::vector<int> nbp_h;
    float *g_raw = nullptr;
    int *nbp = nullptr;
    // adjoint buffers (allocated on first use)
    int *point_win = nullptr, *adj_off = nullptr, *adj_atoms = nullptr;
    double *cvec = nullptr, *lam = nullptr, *grads = nullptr;
    int n_adj_cap = 0;
    double *com = nullptr, *cv = nullptr;
    double *energy = nullptr;  // [n_windows][kECount], allocated on first use
    PointsDev pts{};
    float4 *raw_e = nullptr, *raw_e0 = nullptr;
    float *pts_in = nullptr;
    bool inject = false;
    int *status = nullptr;
    uint32_t *d_step = nullptr;
    unsigned int *d_done = nullptr;
    void *flush = nullptr;
    size_t flush_bytes = 0;

    // scalars shared by all windows
    int n_itypes = 0, n_lj_types = 0, n_g = 0, n_e = 0, n_f = 0;
    float g_r0 = 0, g_dr = 1, e_r0 = 0, e_dr = 1, f_r0 = 0, f_dr = 1, e0 = 0;
    uint64_t seed = 0;

    // graphs
    cudaGraphExec_t graph1 = nullptr, graphN = nullptr;
    std::vector<cudaEvent_t> tev;

    template <typename T>
    T *alloc(size_t n) {
        size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        if (opt.mem_cap && allocated + bytes > opt.mem_cap) throw Fail{ISSPA_ERR_NOMEM};
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Fail{e == cudaErrorMemoryAllocation ? ISSPA_ERR_NOMEM : ISSPA_ERR_CUDA};
        }
        allocs.push_back(p);
        allocated += bytes;
        return static_cast<T *>(p);
    }
    template <typename T>
    T *upload(const std::vector<T> &v) {
        T *p = alloc<T>(v.size());
        // complete before return: later launches go to non-blocking streams
        if (!v.empty()) {
            ck(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
            ck(cudaStreamSynchronize(0));
        }
        return p;
    }
    template <typename T>
    void release(T *&p) {
        if (!p) return;
        auto it = std::find(allocs.begin(), allocs.end(), (void *)p);
        if (it != allocs.end()) allocs.erase(it);
        cudaFree(p);
        p = nullptr;
    }

    // ------------------------------------------------------- work lists
    // Windows in descending size, so the costliest tiles are scheduled first.
    std::vector<int> order;

    static double wave_eff(long long units, long long slots) {
        if (slots <= 0 || units <= 0) return 0.0;
        const double waves = (double)units / (double)slots;
        return waves / std::ceil(waves);
    }
    long long field_tiles_for(int S) const {
        const int tp = field_points_per_block(S);
        long long n = 0;
        for (const WinDev &d : win_h) n += ((long long)d.n_atoms * n_mc + tp - 1) / tp;
        return n;
    }
    long long force_items_for(long long C) const {
        long long n = 0;
        for (const WinDev &d : win_h) n += ((d.n_atoms + 127) / 128) * (((long long)d.n_atoms * n_mc + C - 1) / C);
        return n;
    }
    // Grids of equal-work blocks should fill whole waves of resident blocks:
    // the last, partial wave idles the remaining SMs.
    int default_field_split() const {
        int S = 4;
        double best = -1.0;
        for (int cand : {1, 2, 4, 8, 16}) {
            const double e = wave_eff(field_tiles_for(cand), (long long)n_sms * field_blocks_per_sm(cand));
            if (e > best + 0.02) {
                best = e;
                S = cand;
            }
        }
        return S;
    }
    int default_force_chunk() const {
        const long long slots = (long long)n_sms * std::max(1, force_blocks_per_sm(force_apt));
        double best = -1.0;
        int C = 64;
        for (long long c = 8192; c >= 32; --c) {  // longest chunk (fewest atomics) at equal efficiency
            const long long n = force_items_for(c);
            const double e = n < slots ? 0.5 * (double)n / (double)slots : wave_eff(n, slots);
            if (e > best + 0.005) {
                best = e;
                C = (int)c;
            }
        }
        return C;
    }
    void set_field_split(int S) {
        std::vector<int4> t;
        std::vector<int> base(win_h.size(), 0);
        const int tp = field_points_per_block(S);
        for (int w : order) {
            base[w] = (int)t.size();
            const long long P = (long long)win_h[w].n_atoms * n_mc;
            for (long long p = 0; p < P; p += tp)
                t.push_back(make_int4(w, (int)(win_h[w].point_off + p), (int)std::min<long long>(tp, P - p), 0));
        }
        release(field_tiles);
        field_tiles = upload(t);
        n_field_tiles = (int)t.size();
        field_split = S;
        release(tile_base);
        tile_base = upload(base);
        if (t.size() > tile_flag_cap) {  // fresh stamps are 0, never a pass's stamp
            release(tile_flag);
            tile_flag = alloc<unsigned int>(t.size());
            ck(cudaMemset(tile_flag, 0, t.size() * sizeof(unsigned int)));
            tile_flag_cap = t.size();
        }
    }
    // Force work items: C-point chunks of every window, then (Ct > 0) the last
    // stretch of every window's points in Ct-point chunks, listed after all
    // the long items.  Each item carries a fixed set-up cost (about 2.5 points'
    // worth), so long chunks are cheaper, while the grid's last blocks set
    // the tail; short items at the end fill the SMs the long ones free.  The
    // short stretch is sized to about two waves of resident blocks.
    void set_force_chunk(int C, int Ct = 0) {
        if (Ct >= C) Ct = 0;
        double f = 0.0;  // fraction of each window's points in short chunks
        if (Ct > 0) {
            const long long slots = (long long)n_sms * std::max(1, force_blocks_per_sm(force_apt));
            double point_tiles = 0.0;
            for (const WinDev &d : win_h) point_tiles += (double)d.n_atoms * n_mc * ((d.n_atoms + 127) / 128);
            f = std::min(1.0, 2.0 * (double)slots * Ct / std::max(point_tiles, 1.0));
        }
        std::vector<int4> items, tail;
        std::vector<int2> chunks;
        // chunk-major: blocks that run together read the same point records
        // and add into different atom tiles' accumulators
        auto add = [&](std::vector<int4> &out, int w, long long p0, long long p1, int len) {
            const WinDev &d = win_h[w];
            const int c0 = (int)chunks.size();
            for (long long p = p0; p < p1; p += len)
                chunks.push_back(make_int2((int)(d.point_off + p), (int)std::min<long long>(len, p1 - p)));
            for (int c = c0; c < (int)chunks.size(); ++c)
                for (int a = 0; a < d.n_atoms; a += 128)
                    out.push_back(make_int4(w, d.atom_off + a, std::min(128, d.n_atoms - a), c));
        };
        for (int w : order) {
            const long long P = (long long)win_h[w].n_atoms * n_mc;
            const long long tp = Ct > 0 ? std::min<long long>(P, std::llround(f * (double)P / Ct) * Ct) : 0;
            add(items, w, 0, P - tp, C);
            if (tp > 0) add(tail, w, P - tp, P, Ct);
        }
        items.insert(items.end(), tail.begin(), tail.end());
        release(force_items);
        release(force_chunks);
        force_items = upload(items);
        force_chunks = upload(chunks);
        n_force_items = (int)items.size();
        force_chunk = C;
        force_tail = Ct;
    }

    long long nonbond_items_for(long long J) const {
        long long n = 0;
        for (const WinDev &d : win_h) n += ((d.n_atoms + 127) / 128) * ((d.n_atoms + J - 1) / J);
        return n;
    }
    // The longest partner stretch (fewest stage set-ups and atomics) whose
    // items still fill two waves of resident blocks; 128 when none does.
    int default_nonbond_chunk() const {
        const long long slots = (long long)n_sms * std::max(1, nonbond_blocks_per_sm(n_lj_types));
        for (int J : {4096, 2048, 1024, 768, 512, 384, 256})
            if (nonbond_items_for(J) >= 2 * slots) return J;
        return 128;
    }
    // Nonbond work items, partner-chunk-major: blocks that run together add
    // into different receiving tiles.  Per-stage sums start at multiples of
    // 128 partners from the window's first atom, so J moves no result.
    void set_nonbond_chunk(int J) {
        J = std::max(128, ((J + 127) / 128) * 128);
        std::vector<int4> items;
        std::vector<int> nj;
        for (int w : order) {
            const WinDev &d = win_h[w];
            for (int j = 0; j < d.n_atoms; j += J)
                for (int a = 0; a < d.n_atoms; a += 128) {
                    items.push_back(make_int4(w, d.atom_off + a, std::min(128, d.n_atoms - a), d.atom_off + j));
                    nj.push_back(std::min(J, d.n_atoms - j));
                }
        }
        release(nb_items);
        release(nb_nj);
        nb_items = upload(items);
        nb_nj = upload(nj);
        n_nb_items = (int)items.size();
        nb_chunk = J;
    }

    ~isspa_engine() {
        if (stream) cudaStreamSynchronize(stream);
        if (graph1) cudaGraphExecDestroy(graph1);
        if (graphN) cudaGraphExecDestroy(graphN);
        if (graph_timed) cudaGraphExecDestroy(graph_timed);
        for (const HostStepGraph &h : host_graphs) cudaGraphExecDestroy(h.exec);
        for (auto ev : tev) cudaEventDestroy(ev);
        for (auto ev : kev)
            if (ev) cudaEventDestroy(ev);
        for (cudaEvent_t ev : {ev_fork, ev_join, ev_join2, ev_join3, ev_a, ev_b})
            if (ev) cudaEventDestroy(ev);
        for (void *p : allocs) cudaFree(p);
        if (side) cudaStreamDestroy(side);
        if (side2) cudaStreamDestroy(side2);
        if (side3) cudaStreamDestroy(side3);
        if (stream) cudaStreamDestroy(stream);
    }

    // ---------------------------------------------------------------- args
    FieldArgs field_args() const {
        FieldArgs a{};
        a.vote = field_vote;
        a.tma = field_tma;
        a.pos = pos;
        a.atype = atype;
        a.win = win;
        a.tiles = field_tiles;
        a.n_tiles = opt.isspa_terms ? n_field_tiles : 0;
        a.gtab = gtab;
        a.rmax = rmax;
        a.n_gbins = n_g - 1;
        a.g_r0 = g_r0;
        a.g_dr = g_dr;
        a.g_inv = 1.0f / g_dr;
        a.e_r0 = e_r0;
        a.e_dr = e_dr;
        a.e_inv = 1.0f / e_dr;
        a.e0 = e0;
        a.n_mc = n_mc;
        a.seed_lo = (uint32_t)seed;
        a.seed_hi = (uint32_t)(seed >> 32);
        a.step_ptr = d_step;
        a.pts_in = inject ? pts_in : nullptr;
        a.out = pts;
        a.raw_e = raw_e;
        a.raw_e0 = raw_e0;
        a.terms = opt.isspa_terms;
        a.status = status;
        return a;
    }
    ForceArgs force_args() const {
        ForceArgs a{};
        a.vote = force_vote;
        a.pos = pos;
        a.atype = atype;
        a.win = win;
        a.items = force_items;
        a.chunks = force_chunks;
        a.n_items = opt.isspa_terms ? n_force_items : 0;
        a.pts = pts;
        a.ftab = ftab;
        a.rmax = rmax;
        a.vtot = vtot;
        a.n_f = n_f;
        a.f_r0 = f_r0;
        a.f_dr = f_dr;
        a.f_inv = 1.0f / f_dr;
        a.terms = opt.isspa_terms;
        a.atoms_per_thread = force_apt;
        a.facc = facc;
        a.status = status;
        return a;
    }
    NonbondArgs nonbond_args() const {
        NonbondArgs a{};
        a.pos = pos;
        a.atype = atype;
        a.atom_win = atom_win;
        a.win = win;
        a.items = nb_items;
        a.items_nj = nb_nj;
        a.n_items = opt.nonbond_terms ? n_nb_items : 0;
        a.ljab = ljab;
        a.n_lj_types = n_lj_types;
        a.rmax = rmax;
        a.excl_start = excl_start;
        a.excl = excl;
        a.terms = opt.nonbond_terms;
        a.cut2 = cutoff ? nb_cut2 : INFINITY;
        a.facc = facc;
        a.status = status;
        return a;
    }
    NbListArgs nblist_args() const {
        NbListArgs a{};
        a.pos = pos;
        a.atype = atype;
        a.atom_win = atom_win;
        a.win = win;
        a.wcell = nbl_wcell;
        a.n_atoms = n_atoms;
        a.n_cells = nbl_cells;
        a.ref = nbl_ref;
        a.flag = nbl_flag;
        a.stats = nbl_stats;
        a.cell_of = nbl_cell_of;
        a.cell_count = nbl_cell_count;
        a.cell_start = nbl_cell_start;
        a.cell_cursor = nbl_cell_cursor;
        a.cell_atoms = nbl_cell_atoms;
        a.rows = nbl_rows;
        a.row_n = nbl_row_n;
        a.row_cap = nbl_row_cap;
        a.half_skin2 = nb_half_skin2;
        a.list2 = nb_list2;
        a.cut2 = nb_cut2;
        a.excl_start = excl_start;
        a.excl = excl;
        a.ljab = ljab;
        a.n_lj_types = n_lj_types;
        a.rmax = rmax;
        a.terms = opt.nonbond_terms;
        a.facc = facc;
        a.status = status;
        return a;
    }
    // The nonbond pass: every pair, or in cutoff mode the list check / rebuild
    // and the pairs within the cutoff.
    void enqueue_nonbond(cudaStream_t s) const {
        if (!opt.nonbond_terms) return;
        if (cutoff) {
            const NbListArgs a = nblist_args();
            launch_nblist_build(a, s);
            launch_nblist_pairs(a, s);
        } else {
            launch_nonbond(nonbond_args(), s);
        }
    }
    BondedArgs bonded_args(int b, int an, int d) const {
        BondedArgs a{};
        a.pos = pos;
        a.atom_win = atom_win;
        a.win = win;
        a.bonds = bonds;
        a.n_bonds = n_bonds;
        a.bond_par = bond_par;
        a.angles = angles;
        a.n_angles = n_angles;
        a.angle_par = angle_par;
        a.angle_cs = angle_cs;
        a.dihs = dihs;
        a.dih_type = dih_type;
        a.n_dihs = n_dihs;
        a.dih_par = dih_par;
        a.sc14 = sc14;
        a.ljab = ljab;
        a.atype = atype;
        a.n_lj_types = n_lj_types;
        a.do_bonds = b;
        a.do_angles = an;
        a.do_dihs = d;
        a.facc = facc;
        a.status = status;
        return a;
    }
    UmbrellaArgs umbrella_args() const {
        UmbrellaArgs a{};
        a.pos = pos;
        a.win = win;
        a.us_windows = us_windows;
        a.n_us_windows = n_us;
        a.bias = bias;
        a.mfrac = mfrac;
        a.com = com;
        a.cv = cv;
        a.facc = facc;
        a.status = status;
        return a;
    }
    StateEnergyArgs state_energy_args() const {
        StateEnergyArgs a{};
        a.vel = vel;
        a.facc = facc;
        a.atom_win = atom_win;
        a.win = win;
        a.n_atoms = n_atoms;
        a.us_windows = us_windows;
        a.n_us_windows = n_us;
        a.cv = cv;
        return a;
    }
    LeapfrogArgs leapfrog_args() const {
        LeapfrogArgs a{};
        a.pos = pos;
        a.vel = vel;
        a.force_out = force_out;
        a.facc = facc;
        a.atom_win = atom_win;
        a.win = win;
        a.n_atoms = n_atoms;
        a.seed_lo = (uint32_t)seed;
        a.seed_hi = (uint32_t)(seed >> 32);
        a.step_ptr = d_step;
        a.done_ptr = d_done;
        a.status = status;
        a.ov_epoch = ov_epoch;
        return a;
    }

    IntegratorArgs integrator_args() const {
        IntegratorArgs a{};
        a.bonded = bonded_args(1, 1, 1);
        a.us = umbrella_args();
        a.lf = leapfrog_args();
        a.bias_start = bias_start;
        a.bias_by_atom = bias_by_atom;
        a.usf = usf;
        a.bar = bar;
        return a;
    }
    // Grid of the fused integrator: enough 256-thread blocks for the bonded
    // terms, the atoms and the restrained windows, within the co-resident limit.
    int integrator_grid() const {
        const long long t = integrator_block_threads();
        const long long terms = (long long)n_bonds + n_angles + n_dihs;
        long long g = std::max<long long>({(terms + t - 1) / t, (n_atoms + t - 1) / t, (long long)n_us, 1});
        return (int)std::min<long long>(g, std::max(1, integrator_max_blocks()));
    }

    // The single-kernel step needs split-4 field tiles (128-thread blocks), the
    // LJ table in shared memory, Philox points and the tabulated LJ term on
    // (or no IS-SPA pass); other engines step with separate kernels.
    bool step_kernel_ok() const {
        return n_atoms > 0 && !inject && !cutoff && n_lj_types * n_lj_types <= 4096 &&
               (opt.isspa_terms == 0 || (opt.isspa_terms & 2)) && force_apt == 1;
    }
    StepArgs step_args() const {
        StepArgs a{};
        a.field = field_args();
        a.field.vote = 0;
        a.field.tma = 0;
        a.force = force_args();
        a.force.vote = 0;
        a.nonbond = nonbond_args();
        a.integ = integrator_args();
        return a;
    }
    int step_grid() const {
        const long long t = step_threads();
        const long long terms = (long long)n_bonds + n_angles + n_dihs;
        long long g = std::max<long long>({(long long)(opt.isspa_terms ? n_field_tiles : 0) +
                                               (long long)(opt.nonbond_terms ? n_nb_items : 0),
                                           (long long)(opt.isspa_terms ? n_force_items : 0), (terms + t - 1) / t,
                                           (n_atoms + t - 1) / t, (long long)n_us, 1LL});
        return (int)std::min<long long>(g, std::max(1, step_max_blocks(n_lj_types)));
    }
    // Switches the step integrator; the single-kernel step takes split-4 field
    // tiles (the split in force before it is restored when leaving it).
    int split_before_step = 0;
    void set_integrator(int m) {
        if (m == 3 && !step_kernel_ok()) m = 1;
        if (m == 3 && integrator != 3) {
            split_before_step = field_split;
            if (field_split != 4) set_field_split(4);
        } else if (m != 3 && integrator == 3 && split_before_step && split_before_step != field_split) {
            set_field_split(split_before_step);
        }
        integrator = m;
    }

    // The fused field + force launch needs Philox points, the tabulated LJ term
    // and a field split of 4, 8 or 16; it is offered for windows of at most
    // kFusedMaxAtoms atoms by the autotuner (its force phase adds one set of
    // atomics per atom and field tile).
    static constexpr int kFusedMaxAtoms = 512;
    int max_window_atoms() const {
        int m = 0;
        for (const WinDev &d : win_h) m = std::max(m, d.n_atoms);
        return m;
    }
    bool fused_applies() const { return !inject && (opt.isspa_terms & 2) && n_field_tiles > 0; }
    bool fused_ok() const { return fused_applies() && field_force_fusable(field_split); }
    bool fused() const { return isspa_fused == 1 && fused_ok(); }
    // Force items starting on stamped field tiles: the step's separate passes
    // (launched by isspa_step; the per-call functions keep plain launches)
    bool overlap_ok() const {
        return integrator != 3 && !fused() && opt.isspa_terms && n_field_tiles > 0 && n_force_items > 0;
    }
    bool overlap() const { return force_overlap == 1 && overlap_ok(); }

    // ---------------------------------------------------------- sequences
    void enqueue_isspa(cudaStream_t s, bool raw = false) {
        if (!raw && fused()) {
            launch_field_force(field_args(), force_args(), field_split, s);
            return;
        }
        launch_field(field_args(), field_split, raw, s);
        launch_force(force_args(), s);
    }
    void enqueue_step_serial(cudaStream_t s) {
        launch_bonded(bonded_args(1, 1, 1), s);
        enqueue_isspa(s);
        enqueue_nonbond(s);
        launch_umbrella(umbrella_args(), s);
        launch_leapfrog(leapfrog_args(), s);
    }
    // Which kernels a step launches (the wrappers skip empty work lists).
    bool launches(int k) const {
        const bool one = integrator == 3;
        switch (k) {
            case ISSPA_K_FIELD: return !one && opt.isspa_terms && n_field_tiles > 0;
            case ISSPA_K_FORCE: return !one && !fused() && opt.isspa_terms && n_force_items > 0;
            case ISSPA_K_NONBOND: return !one && opt.nonbond_terms && (cutoff ? n_atoms > 0 : n_nb_items > 0);
            case ISSPA_K_STEP: return one && n_atoms > 0;
            case ISSPA_K_BONDED: return integrator == 1 && n_bonds + n_angles + n_dihs > 0;
            case ISSPA_K_UMBRELLA: return integrator == 1 && n_us > 0;
            case ISSPA_K_LEAPFROG: return integrator == 1 && n_atoms > 0;
            case ISSPA_K_INTEGRATOR: return integrator == 2 && n_atoms > 0;
        }
        return false;
    }
    // Step with independent chains (field -> force or the fused launch;
    // bonded; umbrella; nonbond) on forked streams, all adding into the same
    // accumulator, joined before the update.  With `timed`, CUDA events bracket every kernel on
    // the stream it runs on.
    void enqueue_step_forked(bool timed = false) {
        // External event-record nodes: a plain cudaEventRecord under capture only
        // orders the graph and is never recorded at replay time.
        auto mark = [&](int k, int end, cudaStream_t s) {
            if (timed && launches(k)) ck(cudaEventRecordWithFlags(kev[2 * k + end], s, cudaEventRecordExternal));
        };
        // programmatic launches for the field -> force -> leapfrog chain (not
        // in the event-instrumented copy, whose event nodes sit between them)
        PdlScope pdl(step_pdl == 1 && !timed && integrator != 3);
        if (integrator == 3) {  // the whole step in one cooperative kernel
            mark(ISSPA_K_STEP, 0, stream);
            if (n_atoms > 0) ck(launch_step(step_args(), step_grid(), stream));
            mark(ISSPA_K_STEP, 1, stream);
            return;
        }
        // the umbrella restraint on a branch of its own: with the IS-SPA pass
        // fused, bonded -> restraint in series bounded a restrained small
        // window's step
        const bool us_branch = integrator == 1 && n_us > 0;
        ck(cudaEventRecord(ev_fork, stream));
        ck(cudaStreamWaitEvent(side, ev_fork, 0));
        ck(cudaStreamWaitEvent(side2, ev_fork, 0));
        if (us_branch) ck(cudaStreamWaitEvent(side3, ev_fork, 0));
        mark(ISSPA_K_FIELD, 0, stream);
        if (fused()) {  // one launch for both passes; timed as the field kernel
            launch_field_force(field_args(), force_args(), field_split, stream);
            mark(ISSPA_K_FIELD, 1, stream);
        } else {
            FieldArgs fa = field_args();
            ForceArgs ga = force_args();
            if (overlap()) {
                fa.tile_flag = tile_flag;
                fa.ov_epoch = ov_epoch;
                ga.overlap = 1;
                ga.tile_flag = tile_flag;
                ga.ov_epoch = ov_epoch;
                ga.tile_base = tile_base;
                ga.tile_pts = field_points_per_block(field_split);
            }
            launch_field(fa, field_split, false, stream);
            mark(ISSPA_K_FIELD, 1, stream);
            mark(ISSPA_K_FORCE, 0, stream);
            launch_force(ga, stream);
            mark(ISSPA_K_FORCE, 1, stream);
        }
        if (integrator == 1) {
            mark(ISSPA_K_BONDED, 0, side);
            launch_bonded(bonded_args(1, 1, 1), side);
            mark(ISSPA_K_BONDED, 1, side);
        }
        if (us_branch) {
            mark(ISSPA_K_UMBRELLA, 0, side3);
            launch_umbrella(umbrella_args(), side3);
            mark(ISSPA_K_UMBRELLA, 1, side3);
            ck(cudaEventRecord(ev_join3, side3));
        }
        // nonbond on a third branch: for small systems bonded + restraint and
        // nonbond are each as long as the IS-SPA pass, and in series they
        // were the step's critical path
        mark(ISSPA_K_NONBOND, 0, side2);
        enqueue_nonbond(side2);
        mark(ISSPA_K_NONBOND, 1, side2);
        ck(cudaEventRecord(ev_join, side));
        ck(cudaEventRecord(ev_join2, side2));
        ck(cudaStreamWaitEvent(stream, ev_join, 0));
        ck(cudaStreamWaitEvent(stream, ev_join2, 0));
        if (us_branch) ck(cudaStreamWaitEvent(stream, ev_join3, 0));
        if (integrator == 2) {
            mark(ISSPA_K_INTEGRATOR, 0, stream);
            if (n_atoms > 0) ck(launch_integrator(integrator_args(), integ_grid, stream));
            mark(ISSPA_K_INTEGRATOR, 1, stream);
        } else {
            mark(ISSPA_K_LEAPFROG, 0, stream);
            launch_leapfrog(leapfrog_args(), stream);
            mark(ISSPA_K_LEAPFROG, 1, stream);
        }
    }
    cudaEvent_t kev[2 * ISSPA_K_COUNT] = {};
    cudaGraphExec_t graph_timed = nullptr;
    cudaGraphExec_t capture(int nsteps, bool timed = false) {
        cudaGraph_t g = nullptr;
        ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        try {
            for (int k = 0; k < nsteps; ++k) enqueue_step_forked(timed);
        } catch (...) {
            cudaStreamEndCapture(stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        ck(cudaStreamEndCapture(stream, &g));
        cudaGraphExec_t ex = nullptr;
        // kernel nodes keep the priority of the stream they were captured on
        cudaError_t e = cudaGraphInstantiate(&ex, g, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(g);
        ck(e);
        return ex;
    }
    // isspa_step_host with mapped buffers: copy-in kernel, step and copy-out
    // kernel captured as one graph per set of buffer device addresses (the
    // last few sets kept).  The addresses are resolved through the buffer
    // registry on every call, so a graph is only launched for live buffers.
    struct HostStepGraph {
        const void *key[5];
        cudaGraphExec_t exec;
    };
    std::vector<HostStepGraph> host_graphs;
    cudaGraphExec_t host_step_graph(const void *const key[5], const Copy3Args &in, bool has_in, const Copy3Args &out,
                                    bool has_out) {
        for (const HostStepGraph &h : host_graphs)
            if (std::equal(h.key, h.key + 5, key)) return h.exec;
        cudaGraph_t g = nullptr;
        ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        try {
            if (has_in) launch_copy3(in, stream);
            enqueue_step_forked();
            if (has_out) launch_copy3(out, stream);
        } catch (...) {
            cudaStreamEndCapture(stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        ck(cudaStreamEndCapture(stream, &g));
        cudaGraphExec_t ex = nullptr;
        cudaError_t err = cudaGraphInstantiate(&ex, g, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(g);
        ck(err);
        if (host_graphs.size() >= 4) {
            cudaGraphExecDestroy(host_graphs.front().exec);
            host_graphs.erase(host_graphs.begin());
        }
        HostStepGraph h;
        std::copy(key, key + 5, h.key);
        h.exec = ex;
        host_graphs.push_back(h);
        return ex;
    }
    void invalidate_graphs() {
        if (graph1) cudaGraphExecDestroy(graph1);
        if (graphN) cudaGraphExecDestroy(graphN);
        if (graph_timed) cudaGraphExecDestroy(graph_timed);
        graph1 = graphN = graph_timed = nullptr;
        for (const HostStepGraph &h : host_graphs) cudaGraphExecDestroy(h.exec);
        host_graphs.clear();
    }
    void run_steps(int nsteps) {
        if (!opt.use_graph) {
            for (int k = 0; k < nsteps; ++k) enqueue_step_forked();
            ck(cudaGetLastError());
            return;
        }
        if (!graph1) graph1 = capture(1);
        if (nsteps >= kStepsPerGraph && !graphN) graphN = capture(kStepsPerGraph);
        int k = 0;
        for (; k + kStepsPerGraph <= nsteps; k += kStepsPerGraph) ck(cudaGraphLaunch(graphN, stream));
        for (; k < nsteps; ++k) ck(cudaGraphLaunch(graph1, stream));
    }
};

namespace {

// Effective exclusions of the reference's ascending-list scan
// (nonbond_force_cuda.cu:72-108): partner e_k of atom a is found iff e_k > a
// and no earlier entry of a's list is larger than e_k.
void effective_exclusions(const isspa_host_system &s, std::vector<std::vector<int>> &nb) {
    nb.assign(s.n_atoms, {});
    for (int a = 0; a < s.n_atoms; ++a) {
        int start = a == 0 ? 0 : s.n_excl_cum[a - 1], stop = s.n_excl_cum[a];
        int run_max = INT32_MIN;
        for (int k = start; k < stop; ++k) {
            int e = s.excl_list[k];
            if (e > a && e < s.n_atoms && e >= run_max) {
                nb[a].push_back(e);
                nb[e].push_back(a);
            }
            run_max = std::max(run_max, e);
        }
    }
    for (auto &v : nb) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
}

bool same_force_field(const isspa_host_system &a, const isspa_host_system &b) {
    return a.n_lj_types == b.n_lj_types && a.nb_parm_index == b.nb_parm_index && a.lj_ab == b.lj_ab &&
           a.n_isspa_types == b.n_isspa_types && a.rmax == b.rmax && a.n_g == b.n_g && a.n_e == b.n_e &&
           a.n_f == b.n_f && a.g_table == b.g_table && a.e_table == b.e_table && a.f_table == b.f_table &&
           a.g_r0 == b.g_r0 && a.g_dr == b.g_dr && a.e_r0 == b.e_r0 && a.e_dr == b.e_dr &&
           a.f_r0 == b.f_r0 && a.f_dr == b.f_dr && a.n_mc == b.n_mc && a.seed == b.seed;
}

// Packs the IS-SPA tables for the kernels: g/E as (v_b, v_b+1) pairs per bin of
// the g grid, the force table as (f_k, f_k+1) pairs, both with the reference's
// flat-row semantics (the upper neighbour of a row's last bin is the next
// type's first entry, and zero past the last type).
void pack_isspa_tables(int nt, int ng, int ne, int nf, const std::vector<float> &g, const std::vector<float> &e,
                       const std::vector<float> &f, std::vector<float4> &gtab, std::vector<float2> &ftab) {
    const int pad = std::max({ng, ne, nf}) + 1;
    auto padded = [&](const std::vector<float> &t) {
        std::vector<float> q(t);
        q.resize(t.size() + pad, 0.f);
        return q;
    };
    const std::vector<float> Gp = padded(g), Ep = padded(e), Fp = padded(f);
    gtab.assign((size_t)nt * (ng - 1), make_float4(0.f, 0.f, 0.f, 0.f));
    for (int t = 0; t < nt; ++t)
        for (int b = 0; b < ng - 1; ++b) {
            const size_t gi = (size_t)t * ng + b, ei = (size_t)t * ne + b;
            gtab[(size_t)t * (ng - 1) + b] = make_float4(Gp[gi], Gp[gi + 1], Ep[ei], Ep[ei + 1]);
        }
    ftab.assign((size_t)nt * nf, make_float2(0.f, 0.f));
    for (size_t fi = 0; fi < ftab.size(); ++fi) ftab[fi] = make_float2(Fp[fi], Fp[fi + 1]);
}

// LJ (A, B) for every ordered type pair, from the packed triangle.
void expand_lj(int nlj, const std::vector<int> &nbp, const std::vector<float> &lj_ab, std::vector<float2> &ljab) {
    ljab.resize((size_t)nlj * nlj);
    for (int i = 0; i < nlj * nlj; ++i) ljab[i] = make_float2(lj_ab[2 * nbp[i]], lj_ab[2 * nbp[i] + 1]);
}

void build_nonbond_list(isspa_engine &E);

void build(isspa_engine &E, const std::vector<isspa_host_system> &ws) {
    const isspa_host_system &f0 = ws[0];
    const int W = (int)ws.size();
    E.n_windows = W;
    E.n_mc = f0.n_mc;
    E.seed = f0.seed;
    E.n_itypes = f0.n_isspa_types;
    E.n_lj_types = f0.n_lj_types;
    E.n_g = f0.n_g;
    E.n_e = f0.n_e;
    E.n_f = f0.n_f;
    E.g_r0 = f0.g_r0; E.g_dr = f0.g_dr;
    E.e_r0 = f0.e_r0; E.e_dr = f0.e_dr;
    E.f_r0 = f0.f_r0; E.f_dr = f0.f_dr;
    // e0 = 3/(4 PI rho p0)*(1-1/ep), float as the reference macro (constants.h:13)
    E.e0 = 3.0f / (4.0f * kPi * kRho * kP0) * (1.0f - 1.0f / kEp);

    // ---- concatenated atoms ----
    std::vector<float4> pos, vel;
    std::vector<int2> atype;
    std::vector<int> atom_win;
    std::vector<int4> bonds, angles, dihs;
    std::vector<int> dih_type;
    std::vector<int2> bias;
    std::vector<float> mfrac;
    std::vector<int> us_windows;
    std::vector<std::vector<int>> ex_all;
    E.win_h.resize(W);
    int off = 0;
    long long poff = 0;
    for (int w = 0; w < W; ++w) {
        const isspa_host_system &s = ws[w];
        WinDev &d = E.win_h[w];
        d = WinDev{};
        d.atom_off = off;
        d.n_atoms = s.n_atoms;
        d.point_off = poff;
        d.box = s.box;
        d.hbox = 0.5f * s.box;  // isspa_force_cuda.cu:394
        d.kT = s.kT;
        d.dt = s.dt;
        d.pnu = s.pnu;
        for (int i = 0; i < s.n_atoms; ++i) {
            pos.push_back(make_float4(s.pos[4 * i], s.pos[4 * i + 1], s.pos[4 * i + 2], s.pos[4 * i + 3]));
            vel.push_back(make_float4(s.vel[4 * i], s.vel[4 * i + 1], s.vel[4 * i + 2], s.vel[4 * i + 3]));
            atype.push_back(make_int2(s.lj_type[i], s.isspa_type[i]));
            atom_win.push_back(w);
        }
        for (size_t b = 0; b < s.bond_atoms.size() / 3; ++b)
            bonds.push_back(make_int4(s.bond_atoms[3 * b] + off, s.bond_atoms[3 * b + 1] + off,
                                      s.bond_atoms[3 * b + 2], 0));
        for (size_t b = 0; b < s.angle_atoms.size() / 4; ++b)
            angles.push_back(make_int4(s.angle_atoms[4 * b] + off, s.angle_atoms[4 * b + 1] + off,
                                       s.angle_atoms[4 * b + 2] + off, s.angle_atoms[4 * b + 3]));
        for (size_t b = 0; b < s.dih_types.size(); ++b) {
            const int *a = &s.dih_atoms[4 * b];
            const bool do14 = a[2] > 0 && a[3] > 0;  // dih_force_cuda.cu:60
            dihs.push_back(make_int4(std::abs(a[0]) + off, std::abs(a[1]) + off, std::abs(a[2]) + off,
                                     std::abs(a[3]) + off));
            dih_type.push_back(s.dih_types[b] | (do14 ? 0x40000000 : 0));
        }
        if (s.us_on) {
            d.us_on = 1;
            d.bias_off = (int)bias.size();
            d.n_bias = (int)s.bias_list.size() / 2;
            d.us_k = s.us_k;
            d.us_x0 = s.us_x0;
            // us_class.cpp:136-152: mass fractions in float
            float tot[2] = {0.f, 0.f};
            for (int b = 0; b < d.n_bias; ++b) tot[s.bias_list[2 * b + 1]] += s.raw_mass[s.bias_list[2 * b]];
            for (int b = 0; b < d.n_bias; ++b) {
                int a = s.bias_list[2 * b], g = s.bias_list[2 * b + 1];
                bias.push_back(make_int2(a + off, g));
                mfrac.push_back(s.raw_mass[a] / tot[g]);
            }
            if (!(tot[0] > 0.f) || !(tot[1] > 0.f)) throw Fail{ISSPA_ERR_ARG};
            us_windows.push_back(w);
        }
        std::vector<std::vector<int>> ex;
        effective_exclusions(s, ex);
        for (auto &v : ex) {
            for (int &j : v) j += off;
            ex_all.push_back(std::move(v));
        }
        off += s.n_atoms;
        poff += (long long)s.n_atoms * s.n_mc;
    }
    E.n_atoms = off;
    E.n_points = poff;
    E.n_bonds = (int)bonds.size();
    E.n_angles = (int)angles.size();
    E.n_dihs = (int)dihs.size();
    E.n_us = (int)us_windows.size();

    // ---- force-field tables ----
    const int nt = E.n_itypes;
    std::vector<float4> gtab;
    std::vector<float2> ftab;
    pack_isspa_tables(nt, f0.n_g, f0.n_e, f0.n_f, f0.g_table, f0.e_table, f0.f_table, gtab, ftab);
    std::vector<float> vtot(nt);
    for (int t = 0; t < nt; ++t) {
        // isspa_class.cpp:41 (double arithmetic, stored as float)
        double r = f0.rmax[t];
        vtot[t] = (float)(4.0 / 3.0 * (double)kPi * r * r * r * 0.0074 / (double)(float)f0.n_mc);
    }
    std::vector<float2> ljab;
    expand_lj(f0.n_lj_types, f0.nb_parm_index, f0.lj_ab, ljab);
    std::vector<int> ex_start(E.n_atoms + 1, 0), ex_flat;
    for (int i = 0; i < E.n_atoms; ++i) {
        ex_start[i] = (int)ex_flat.size();
        ex_flat.insert(ex_flat.end(), ex_all[i].begin(), ex_all[i].end());
    }
    ex_start[E.n_atoms] = (int)ex_flat.size();
    std::vector<float2> bond_par, angle_par, sc14;
    std::vector<float4> dih_par;
    // per-window bonded parameter tables may differ: concatenate with offsets
    {
        int bo = 0, ao = 0, dofs = 0;
        size_t bi = 0, ai = 0, di = 0;
        for (int w = 0; w < W; ++w) {
            const isspa_host_system &s = ws[w];
            for (int t = 0; t < s.n_bond_types; ++t) bond_par.push_back(make_float2(s.bond_params[2 * t], s.bond_params[2 * t + 1]));
            for (int t = 0; t < s.n_angle_types; ++t) angle_par.push_back(make_float2(s.angle_params[2 * t], s.angle_params[2 * t + 1]));
            for (int t = 0; t < s.n_dih_types; ++t) {
                dih_par.push_back(make_float4(s.dih_params[4 * t], s.dih_params[4 * t + 1], s.dih_params[4 * t + 2], 0.f));
                sc14.push_back(make_float2(s.scaled14[2 * t], s.scaled14[2 * t + 1]));
            }
            for (size_t b = 0; b < s.bond_atoms.size() / 3; ++b) bonds[bi++].z += bo;
            for (size_t b = 0; b < s.angle_atoms.size() / 4; ++b) angles[ai++].w += ao;
            for (size_t b = 0; b < s.dih_types.size(); ++b) dih_type[di++] += dofs;
            bo += s.n_bond_types;
            ao += s.n_angle_types;
            dofs += s.n_dih_types;
        }
    }

    // ---- work lists ----
    E.order.resize(W);
    for (int w = 0; w < W; ++w) E.order[w] = w;
    std::stable_sort(E.order.begin(), E.order.end(),
                     [&](int a, int b) { return ws[a].n_atoms > ws[b].n_atoms; });
    if (E.n_points > INT32_MAX) throw Fail{ISSPA_ERR_UNSUPPORTED};
    int dev = 0, sms = 0;
    ck(cudaGetDevice(&dev));
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    E.n_sms = sms;
    int S = E.opt.field_split;
    if (S != 1 && S != 2 && S != 4 && S != 8 && S != 16) S = E.default_field_split();
    E.set_field_split(S);
    E.field_vote = E.opt.field_vote == 1 ? 1 : 0;
    E.field_tma = E.opt.field_tma == 1 ? 1 : 0;
    E.step_pdl = E.opt.step_pdl == 1 ? 1 : 0;
    E.isspa_fused = E.opt.isspa_fused == 1 ? 1 : 0;
    E.force_overlap = E.opt.force_overlap == 1 ? 1 : 0;
    E.force_vote = E.opt.force_vote == 1 ? 1 : 0;
    E.force_apt = E.opt.force_atoms_per_thread == 2 ? 2 : 1;
    E.set_force_chunk(E.opt.force_chunk > 0 ? E.opt.force_chunk : E.default_force_chunk(),
                      std::max(0, E.opt.force_tail_chunk));
    // nonbond items: 128 i-atoms x J partners (J a multiple of 128)
    E.set_nonbond_chunk(E.opt.nonbond_chunk > 0 ? ((E.opt.nonbond_chunk + 127) / 128) * 128
                                                : E.default_nonbond_chunk());

    // ---- upload ----
    E.pos = E.upload(pos);
    E.vel = E.upload(vel);
    E.force_out = E.alloc<float4>(E.n_atoms);
    E.facc = E.alloc<unsigned long long>(3 * (size_t)E.n_atoms);
    ck(cudaMemset(E.facc, 0, 3 * sizeof(unsigned long long) * E.n_atoms));
    ck(cudaMemset(E.force_out, 0, sizeof(float4) * E.n_atoms));
    E.atype = E.upload(atype);
    E.atom_win = E.upload(atom_win);
    E.win = E.upload(E.win_h);
    E.gtab = E.upload(gtab);
    E.ftab = E.upload(ftab);
    E.rmax = E.upload(f0.rmax);
    E.vtot = E.upload(vtot);
    E.ljab = E.upload(ljab);
    E.excl_start = E.upload(ex_start);
    E.excl = E.upload(ex_flat);
    E.bonds = E.upload(bonds);
    E.angles = E.upload(angles);
    E.dihs = E.upload(dihs);
    E.dih_type = E.upload(dih_type);
    E.bond_par = E.upload(bond_par);
    E.angle_par = E.upload(angle_par);
    {
        // cos / sin of each equilibrium angle (the float parameter, exactly)
        // as double-float pairs for the bend theta - theta0
        std::vector<float4> cs(angle_par.size());
        for (size_t t = 0; t < angle_par.size(); ++t) {
            const double th = (double)angle_par[t].y, c = std::cos(th), sn = std::sin(th);
            const float ch = (float)c, sh = (float)sn;
            cs[t] = make_float4(ch, (float)(c - (double)ch), sh, (float)(sn - (double)sh));
        }
        E.angle_cs = E.upload(cs);
    }
    E.dih_par = E.upload(dih_par);
    E.sc14 = E.upload(sc14);
    E.us_windows = E.upload(us_windows);
    E.bias = E.upload(bias);
    E.mfrac = E.upload(mfrac);
    // host copies kept for the adjoint and for table updates
    E.bias_h = bias;
    E.mfrac_h = mfrac;
    E.nbp_h = f0.nb_parm_index;
    E.lj_ab_h = f0.lj_ab;
    E.g_raw_h = f0.g_table;
    E.e_raw_h = f0.e_table;
    E.f_raw_h = f0.f_table;
    E.g_raw = E.upload(f0.g_table);
    E.nbp = E.upload(f0.nb_parm_index);
    E.com = E.alloc<double>(6 * (size_t)W);
    E.cv = E.alloc<double>(W);
    ck(cudaMemset(E.com, 0, sizeof(double) * 6 * W));
    ck(cudaMemset(E.cv, 0, sizeof(double) * W));
    E.pts.q0 = E.alloc<float4>(E.n_points);
    E.pts.q1 = E.alloc<float4>(E.n_points);
    E.pts.q2 = E.alloc<float4>(E.n_points);
    E.pts.q3 = E.alloc<float4>(E.n_points);
    E.pts.q4 = E.alloc<float4>(E.n_points);
    // restraint entries grouped by atom, for the fused integrator
    {
        std::vector<int> start(E.n_atoms + 1, 0), by_atom(bias.size());
        for (const int2 &b : bias) ++start[b.x + 1];
        for (int i = 0; i < E.n_atoms; ++i) start[i + 1] += start[i];
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (size_t b = 0; b < bias.size(); ++b) by_atom[fill[bias[b].x]++] = (int)b;
        E.bias_start = E.upload(start);
        E.bias_by_atom = E.upload(by_atom);
    }
    E.usf = E.alloc<double2>(2 * (size_t)W);
    E.bar = E.alloc<unsigned int>(2);
    ck(cudaMemset(E.bar, 0, 2 * sizeof(unsigned int)));
    E.integrator = 1;
    E.cutoff = E.opt.nonbond_cutoff > 0.f;  // (its list is built below) no single-kernel step
    if (E.opt.integrator == 2 || E.opt.integrator == 3) E.set_integrator(E.opt.integrator);
    E.integ_grid = E.integrator_grid();
    E.status = E.alloc<int>(1);
    E.d_step = E.alloc<uint32_t>(1);
    E.d_done = E.alloc<unsigned int>(1);
    E.ov_epoch = E.alloc<unsigned int>(1);
    ck(cudaMemset(E.ov_epoch, 0, sizeof(unsigned int)));
    ck(cudaMemset(E.status, 0, sizeof(int)));
    ck(cudaMemset(E.d_step, 0, sizeof(uint32_t)));
    ck(cudaMemset(E.d_done, 0, sizeof(unsigned int)));
    if (E.opt.nonbond_cutoff > 0.f) build_nonbond_list(E);
}

// Cutoff mode of the nonbond pass: per-window cell grids (cells at least
// 1.0001 (cutoff + skin) on a side, at most about 8 per atom, the whole window
// as one cell below 3 per edge), the list buffers, and the row capacity -- the
// option, or 1.5 x the fullest row of the starting configuration + 32 (at most
// the largest window), found by a counting pass of the list build.
void build_nonbond_list(isspa_engine &E) {
    const float rc = E.opt.nonbond_cutoff;
    const float skin = E.opt.nonbond_skin > 0.f ? E.opt.nonbond_skin : 2.0f;
    const float rl = rc + skin;
    E.cutoff = true;
    E.nb_cut2 = rc * rc;
    E.nb_list2 = rl * rl;
    // rebuild beyond 0.499 skin (not 0.5): a margin far above the rounding of
    // the FP32 displacement and distance checks
    const float half = 0.499f * skin;
    E.nb_half_skin2 = half * half;
    const int W = E.n_windows;
    std::vector<int4> wcell(W);
    long long cells = 0;
    int max_n = 1;
    for (int w = 0; w < W; ++w) {
        const WinDev &d = E.win_h[w];
        max_n = std::max(max_n, d.n_atoms);
        const double geo = std::floor((double)d.box / (1.0001 * (double)rl));
        const double cap = std::floor(std::cbrt(8.0 * std::max(d.n_atoms, 1)));
        const int nc = std::min(geo, cap) >= 3.0 ? (int)std::min(geo, cap) : 1;
        const float scale = (float)nc / d.box;
        int bits = 0;
        std::memcpy(&bits, &scale, sizeof bits);
        wcell[w] = make_int4((int)cells, nc, bits, 0);
        cells += (long long)nc * nc * nc;
    }
    if (cells > INT32_MAX / 2) throw Fail{ISSPA_ERR_UNSUPPORTED};
    E.nbl_cells = (int)cells;
    const size_t N = (size_t)E.n_atoms;
    E.nbl_wcell = E.upload(wcell);
    E.nbl_ref = E.alloc<float4>(N);
    E.nbl_flag = E.alloc<int>(1);
    E.nbl_stats = E.alloc<int>(2);
    E.nbl_cell_of = E.alloc<int>(N);
    E.nbl_cell_count = E.alloc<int>(cells);
    E.nbl_cell_start = E.alloc<int>(cells + 1);
    E.nbl_cell_cursor = E.alloc<int>(cells);
    E.nbl_cell_atoms = E.alloc<int>(N);
    E.nbl_row_n = E.alloc<int>(N);
    ck(cudaMemset(E.nbl_cell_count, 0, sizeof(int) * cells));
    auto reset = [&] {  // NaN reference positions: the next check rebuilds
        ck(cudaMemset(E.nbl_ref, 0xff, sizeof(float4) * N));
        ck(cudaMemset(E.nbl_flag, 0, sizeof(int)));
        ck(cudaMemset(E.nbl_stats, 0, 2 * sizeof(int)));
    };
    reset();
    int cap = E.opt.nonbond_list_max;
    if (cap <= 0) {
        NbListArgs a = E.nblist_args();
        a.rows = nullptr;
        launch_nblist_build(a, E.stream);
        ck(cudaGetLastError());
        int st[2] = {0, 0};
        ck(cudaMemcpyAsync(st, E.nbl_stats, sizeof st, cudaMemcpyDeviceToHost, E.stream));
        ck(cudaStreamSynchronize(E.stream));
        cap = ((st[1] * 3 / 2 + 32 + 31) / 32) * 32;
        reset();
    }
    E.nbl_row_cap = std::max(1, std::min(cap, max_n));
    E.nbl_rows = E.alloc<int>(N * (size_t)E.nbl_row_cap);
}

int guard(isspa_engine *e) {
    if (!e) return ISSPA_ERR_ARG;
    return cudaSetDevice(e->device) == cudaSuccess ? ISSPA_OK : ISSPA_ERR_CUDA;
}

template <typename F>
int run_guarded(F &&f) {
    try {
        f();
        return cudaGetLastError() == cudaSuccess ? ISSPA_OK : ISSPA_ERR_CUDA;
    } catch (const Fail &x) {
        cudaGetLastError();
        return x.code;
    } catch (const std::bad_alloc &) {
        return ISSPA_ERR_NOMEM;
    }
}

// Times `f` with CUDA events on the engine stream when ms_out is given.
template <typename F>
int timed_call(isspa_engine *e, float *ms_out, F &&f) {
    int rc = guard(e);
    if (rc) return rc;
    return run_guarded([&] {
        if (ms_out) ck(cudaEventRecord(e->ev_a, e->stream));
        f();
        ck(cudaGetLastError());
        if (ms_out) {
            ck(cudaEventRecord(e->ev_b, e->stream));
            ck(cudaEventSynchronize(e->ev_b));
            ck(cudaEventElapsedTime(ms_out, e->ev_a, e->ev_b));
        }
    });
}

}  // namespace

extern "C" {

const char *isspa_strerror(int s) {
    switch (s) {
        case ISSPA_OK: return "ok";
        case ISSPA_ERR_ARG: return "invalid argument";
        case ISSPA_ERR_IO: return "file could not be opened";
        case ISSPA_ERR_PARSE: return "malformed input file";
        case ISSPA_ERR_CUDA: return "CUDA runtime error";
        case ISSPA_ERR_NOMEM: return "out of device memory (or over the engine memory cap)";
        case ISSPA_ERR_BOUNDS: return "device bounds check tripped";
        case ISSPA_ERR_TIMEOUT: return "bounded device wait timed out";
        case ISSPA_ERR_NONFINITE: return "non-finite force or coordinate";
        case ISSPA_ERR_UNSUPPORTED: return "input outside what the engine supports";
        case ISSPA_ERR_STATE: return "call not valid in the engine state";
        case ISSPA_ERR_OVERFLOW: return "force outside the fixed-point range";
        case ISSPA_ERR_LIST_FULL: return "a neighbour-list row outgrew its capacity";
        default: return "unknown status";
    }
}

int isspa_device_count(int *count) {
    if (!count) return ISSPA_ERR_ARG;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *count = n;
    return ISSPA_OK;
}

void isspa_default_options(isspa_engine_options *o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->isspa_terms = 7;
    o->nonbond_terms = 7;
    o->use_graph = 1;
}

int isspa_engine_create(const isspa_system_desc *windows, int n_windows, const isspa_engine_options *opt,
                        isspa_engine **out) {
    if (!windows || n_windows <= 0 || !out) return ISSPA_ERR_ARG;
    *out = nullptr;
    std::vector<isspa_host_system> ws(n_windows);
    for (int w = 0; w < n_windows; ++w) {
        int rc = host_system_from_desc(windows[w], ws[w]);
        if (rc) return rc;
        if (w && !same_force_field(ws[0], ws[w])) return ISSPA_ERR_UNSUPPORTED;
    }
    std::unique_ptr<isspa_engine> e;
    try {
        e.reset(new isspa_engine());
    } catch (...) {
        return ISSPA_ERR_NOMEM;
    }
    if (opt) e->opt = *opt;
    else isspa_default_options(&e->opt);
    // 0 selects every term; ISSPA_TERMS_NONE switches the pass off (mask 0)
    if (e->opt.isspa_terms < 0) e->opt.isspa_terms = 0;
    else if (e->opt.isspa_terms == 0) e->opt.isspa_terms = 7;
    if (e->opt.nonbond_terms < 0) e->opt.nonbond_terms = 0;
    else if (e->opt.nonbond_terms == 0) e->opt.nonbond_terms = 7;
    if (!(e->opt.nonbond_cutoff >= 0.f) || !(e->opt.nonbond_skin >= 0.f) || e->opt.nonbond_list_max < 0 ||
        std::isinf(e->opt.nonbond_cutoff) || std::isinf(e->opt.nonbond_skin) || e->opt.step_pdl < 0 ||
        e->opt.step_pdl > 2 || e->opt.isspa_fused < 0 || e->opt.isspa_fused > 2 || e->opt.force_overlap < 0 ||
        e->opt.force_overlap > 2)
        return ISSPA_ERR_ARG;
    if (cudaGetDevice(&e->device) != cudaSuccess) {
        cudaGetLastError();
        return ISSPA_ERR_CUDA;
    }
    int rc = run_guarded([&] {
        ck(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        // the side branches (bonded and umbrella; nonbond: a few hundred
        // blocks) at the highest priority, so their blocks are dispatched ahead
        // of the field and force grids' queued blocks instead of after them
        int prio_low = 0, prio_high = 0;
        ck(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
        ck(cudaStreamCreateWithPriority(&e->side, cudaStreamNonBlocking, prio_high));
        ck(cudaStreamCreateWithPriority(&e->side2, cudaStreamNonBlocking, prio_high));
        ck(cudaStreamCreateWithPriority(&e->side3, cudaStreamNonBlocking, prio_high));
        for (cudaEvent_t *ev : {&e->ev_fork, &e->ev_join, &e->ev_join2, &e->ev_join3})
            ck(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
        ck(cudaEventCreate(&e->ev_a));
        ck(cudaEventCreate(&e->ev_b));
        build(*e, ws);
        ck(cudaDeviceSynchronize());
    });
    if (rc) return rc;
    *out = e.release();
    return ISSPA_OK;
}

void isspa_engine_destroy(isspa_engine *e) {
    if (!e) return;
    cudaSetDevice(e->device);
    delete e;
}

int isspa_engine_info(const isspa_engine *e, int *nw, int *na, long long *np) {
    if (!e) return ISSPA_ERR_ARG;
    if (nw) *nw = e->n_windows;
    if (na) *na = e->n_atoms;
    if (np) *np = e->n_points;
    return ISSPA_OK;
}

int isspa_engine_shapes(const isspa_engine *e, int shape[ISSPA_SHAPE_COUNT]) {
    if (!e || !shape) return ISSPA_ERR_ARG;
    shape[0] = e->field_split;
    shape[1] = e->n_field_tiles;
    shape[2] = e->force_chunk;
    shape[3] = e->n_force_items;
    shape[4] = e->n_nb_items;
    shape[5] = e->nb_chunk;
    shape[6] = e->n_sms;
    shape[7] = e->force_apt;
    shape[8] = e->force_tail;
    shape[9] = e->field_vote;
    shape[10] = e->force_apt == 1 ? e->force_vote : 0;
    shape[11] = e->integrator;
    shape[12] = e->field_tma;
    shape[13] = e->cutoff ? e->nbl_row_cap : 0;
    shape[14] = e->cutoff ? e->nbl_cells : 0;
    shape[15] = e->step_pdl;
    shape[16] = e->fused() ? 1 : 0;
    shape[17] = e->overlap() ? 1 : 0;
    return ISSPA_OK;
}

int isspa_set_tables(isspa_engine *e, const float *g_table, const float *e_table, const float *f_table,
                     const float *lj_ab) {
    int rc = guard(e);
    if (rc) return rc;
    return run_guarded([&] {
        const int nt = e->n_itypes, nlj = e->n_lj_types;
        if (g_table) e->g_raw_h.assign(g_table, g_table + (size_t)nt * e->n_g);
        if (e_table) e->e_raw_h.assign(e_table, e_table + (size_t)nt * e->n_e);
        if (f_table) e->f_raw_h.assign(f_table, f_table + (size_t)nt * e->n_f);
        if (lj_ab) e->lj_ab_h.assign(lj_ab, lj_ab + (size_t)nlj * (nlj + 1));
        for (float v : e->g_raw_h) if (!std::isfinite(v)) throw Fail{ISSPA_ERR_ARG};
        for (float v : e->e_raw_h) if (!std::isfinite(v)) throw Fail{ISSPA_ERR_ARG};
        for (float v : e->f_raw_h) if (!std::isfinite(v)) throw Fail{ISSPA_ERR_ARG};
        for (float v : e->lj_ab_h) if (!std::isfinite(v)) throw Fail{ISSPA_ERR_ARG};
        std::vector<float4> gtab;
        std::vector<float2> ftab, ljab;
        pack_isspa_tables(nt, e->n_g, e->n_e, e->n_f, e->g_raw_h, e->e_raw_h, e->f_raw_h, gtab, ftab);
        expand_lj(nlj, e->nbp_h, e->lj_ab_h, ljab);
        // ordered on the engine's non-blocking stream, before any later launch
        ck(cudaStreamSynchronize(e->stream));
        ck(cudaMemcpyAsync(e->gtab, gtab.data(), sizeof(float4) * gtab.size(), cudaMemcpyHostToDevice, e->stream));
        ck(cudaMemcpyAsync(e->ftab, ftab.data(), sizeof(float2) * ftab.size(), cudaMemcpyHostToDevice, e->stream));
        ck(cudaMemcpyAsync(e->ljab, ljab.data(), sizeof(float2) * ljab.size(), cudaMemcpyHostToDevice, e->stream));
        ck(cudaMemcpyAsync(e->g_raw, e->g_raw_h.data(), sizeof(float) * e->g_raw_h.size(), cudaMemcpyHostToDevice,
                           e->stream));
        ck(cudaStreamSynchronize(e->stream));
    });
}

int isspa_adjoint_mean_force(isspa_engine *e, int n_frames, const float *frames, const uint32_t *steps, double *J,
                             double *dJ_df, double *dJ_dg, double *dJ_dA, double *dJ_dB) {
    if (!e || n_frames <= 0 || !steps) return ISSPA_ERR_ARG;
    int rc = guard(e);
    if (rc) return rc;
    // the gradient kernels differentiate the full force (every term)
    if ((e->opt.isspa_terms & 7) != 7 || (e->opt.nonbond_terms & 7) != 7) return ISSPA_ERR_STATE;
    // its pair kernels differentiate every pair, not the truncated force
    if (e->cutoff) return ISSPA_ERR_UNSUPPORTED;
    const int W = e->n_windows, N = e->n_atoms;
    const long long P = e->n_points;
    const long long nF = (long long)e->n_itypes * e->n_f, nG = (long long)e->n_itypes * e->n_g;
    const int ntt = e->n_lj_types * (e->n_lj_types + 1) / 2;
    const long long per_w = nF + nG + 2LL * ntt;
    std::vector<float4> saved(N);
    uint32_t saved_step = 0;
    rc = run_guarded([&] {
        if (!e->raw_e) {
            e->raw_e = e->alloc<float4>(P);
            e->raw_e0 = e->alloc<float4>(P);
        }
        if (!e->point_win) {
            std::vector<int> pw(P);
            for (int w = 0; w < W; ++w)
                for (long long p = 0; p < (long long)e->win_h[w].n_atoms * e->n_mc; ++p) pw[e->win_h[w].point_off + p] = w;
            e->point_win = e->upload(pw);
            e->cvec = e->alloc<double>(3 * (size_t)N);
            e->lam = e->alloc<double>(P);
            e->grads = e->alloc<double>((size_t)W * per_w);
            e->adj_off = e->alloc<int>(W + 1);
            e->adj_atoms = e->alloc<int>(std::max<size_t>(1, e->bias_h.size()));
        }
        // Every copy below is ordered on the engine's (non-blocking) stream: a
        // legacy-stream cudaMemcpy does not wait for the previous frame's
        // adjoint kernels, and would overwrite positions and weights under them.
        ck(cudaStreamSynchronize(e->stream));
        ck(cudaMemcpyAsync(saved.data(), e->pos, sizeof(float4) * N, cudaMemcpyDeviceToHost, e->stream));
        ck(cudaMemcpyAsync(&saved_step, e->d_step, sizeof saved_step, cudaMemcpyDeviceToHost, e->stream));
        ck(cudaMemsetAsync(e->grads, 0, sizeof(double) * (size_t)W * per_w, e->stream));
        ck(cudaStreamSynchronize(e->stream));
        std::vector<double> Jw(W, 0.0), cvec(3 * (size_t)N), facc(3 * (size_t)N);
        std::vector<long long> acc(3 * (size_t)N);
        for (int f = 0; f < n_frames; ++f) {
            const float4 *X = frames ? reinterpret_cast<const float4 *>(frames) + (size_t)f * N : saved.data();
            if (frames) ck(cudaMemcpyAsync(e->pos, X, sizeof(float4) * N, cudaMemcpyHostToDevice, e->stream));
            ck(cudaMemcpyAsync(e->d_step, &steps[f], sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
            // weights c_i = +-n/2 on the two restraint groups of each window
            std::fill(cvec.begin(), cvec.end(), 0.0);
            std::vector<int> off(W + 1, 0), atoms;
            for (int w = 0; w < W; ++w) {
                off[w] = (int)atoms.size();
                const WinDev &d = e->win_h[w];
                if (!d.us_on) continue;
                double c[2][3] = {{0, 0, 0}, {0, 0, 0}};
                for (int b = 0; b < d.n_bias; ++b) {
                    const int2 bl = e->bias_h[d.bias_off + b];
                    const double m = e->mfrac_h[d.bias_off + b];
                    c[bl.y][0] += m * X[bl.x].x;
                    c[bl.y][1] += m * X[bl.x].y;
                    c[bl.y][2] += m * X[bl.x].z;
                }
                double n[3], nn = 0.0;
                for (int k = 0; k < 3; ++k) {
                    double v = c[0][k] - c[1][k];
                    if (v > 0.5 * d.box) v -= d.box;
                    else if (v < -0.5 * d.box) v += d.box;
                    n[k] = v;
                    nn += v * v;
                }
                nn = std::sqrt(nn);
                for (int b = 0; b < d.n_bias; ++b) {
                    const int2 bl = e->bias_h[d.bias_off + b];
                    const double sgn = bl.y == 0 ? 0.5 : -0.5;
                    for (int k = 0; k < 3; ++k) cvec[3 * (size_t)bl.x + k] += sgn * n[k] / nn;
                    if (std::find(atoms.begin() + off[w], atoms.end(), bl.x) == atoms.end()) atoms.push_back(bl.x);
                }
            }
            off[W] = (int)atoms.size();
            ck(cudaMemcpyAsync(e->cvec, cvec.data(), sizeof(double) * cvec.size(), cudaMemcpyHostToDevice, e->stream));
            ck(cudaMemcpyAsync(e->adj_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, e->stream));
            if (!atoms.empty())
                ck(cudaMemcpyAsync(e->adj_atoms, atoms.data(), sizeof(int) * atoms.size(), cudaMemcpyHostToDevice,
                                   e->stream));
            // the value: every non-restraint force of the frame, projected
            ck(cudaMemsetAsync(e->facc, 0, 3 * sizeof(unsigned long long) * N, e->stream));
            launch_bonded(e->bonded_args(1, 1, 1), e->stream);
            launch_field(e->field_args(), e->field_split, true, e->stream);
            launch_force(e->force_args(), e->stream);
            launch_nonbond(e->nonbond_args(), e->stream);
            ck(cudaGetLastError());
            ck(cudaMemcpyAsync(acc.data(), e->facc, sizeof(long long) * acc.size(), cudaMemcpyDeviceToHost, e->stream));
            ck(cudaStreamSynchronize(e->stream));
            for (int w = 0; w < W; ++w) {
                const WinDev &d = e->win_h[w];
                for (int i = d.atom_off; i < d.atom_off + d.n_atoms; ++i)
                    for (int k = 0; k < 3; ++k) Jw[w] += cvec[3 * (size_t)i + k] * (double)acc[3 * (size_t)i + k] * kFixInv;
            }
            // the gradient
            AdjointArgs a{};
            a.pos = e->pos;
            a.atype = e->atype;
            a.win = e->win;
            a.atom_win = e->atom_win;
            a.n_points = P;
            a.point_win = e->point_win;
            a.raw_e = e->raw_e;
            a.raw_e0 = e->raw_e0;
            a.q0 = e->pts.q0;
            a.adj_off = e->adj_off;
            a.adj_atoms = e->adj_atoms;
            a.n_adj = (int)atoms.size();
            a.cvec = e->cvec;
            a.rmax = e->rmax;
            a.vtot = e->vtot;
            a.f_r0 = e->f_r0;
            a.f_dr = e->f_dr;
            a.f_inv = 1.0f / e->f_dr;
            a.n_f = e->n_f;
            a.ftab = e->ftab;
            a.n_ftab = nF;
            a.dJ_df = e->grads;
            a.lam = e->lam;
            a.g_table = e->g_raw;
            a.n_g = e->n_g;
            a.g_r0 = e->g_r0;
            a.g_dr = e->g_dr;
            a.g_inv = 1.0f / e->g_dr;
            a.n_gtab = nG;
            a.dJ_dg = e->grads + (size_t)W * nF;
            a.n_mc = e->n_mc;
            a.excl_start = e->excl_start;
            a.excl = e->excl;
            a.nbp = e->nbp;
            a.n_lj_types = e->n_lj_types;
            a.n_ljtab = ntt;
            a.dJ_dA = e->grads + (size_t)W * (nF + nG);
            a.dJ_dB = e->grads + (size_t)W * (nF + nG + ntt);
            a.dihs = e->dihs;
            a.dih_type = e->dih_type;
            a.n_dihs = e->n_dihs;
            a.sc14 = e->sc14;
            launch_adjoint(a, e->stream);
            ck(cudaGetLastError());
            // the next frame rewrites cvec/off/atoms and the device positions
            ck(cudaStreamSynchronize(e->stream));
        }
        std::vector<double> g((size_t)W * per_w);
        ck(cudaMemcpyAsync(g.data(), e->grads, sizeof(double) * g.size(), cudaMemcpyDeviceToHost, e->stream));
        ck(cudaStreamSynchronize(e->stream));
        const double inv = 1.0 / n_frames;
        for (int w = 0; w < W; ++w) {
            if (J) J[w] = Jw[w] * inv;
            for (long long k = 0; k < nF; ++k)
                if (dJ_df) dJ_df[w * nF + k] = g[(size_t)w * nF + k] * inv;
            for (long long k = 0; k < nG; ++k)
                if (dJ_dg) dJ_dg[w * nG + k] = g[(size_t)W * nF + (size_t)w * nG + k] * inv;
            for (int k = 0; k < ntt; ++k) {
                if (dJ_dA) dJ_dA[(size_t)w * ntt + k] = g[(size_t)W * (nF + nG) + (size_t)w * ntt + k] * inv;
                if (dJ_dB) dJ_dB[(size_t)w * ntt + k] = g[(size_t)W * (nF + nG + ntt) + (size_t)w * ntt + k] * inv;
            }
        }
        // restore the engine's state
        ck(cudaMemcpyAsync(e->pos, saved.data(), sizeof(float4) * N, cudaMemcpyHostToDevice, e->stream));
        ck(cudaMemcpyAsync(e->d_step, &saved_step, sizeof saved_step, cudaMemcpyHostToDevice, e->stream));
        ck(cudaMemsetAsync(e->facc, 0, 3 * sizeof(unsigned long long) * N, e->stream));
        ck(cudaStreamSynchronize(e->stream));
    });
    return rc;
}

static_assert(kECount == ISSPA_E_COUNT && kEVirial == ISSPA_E_VIRIAL && kEUmbrella == ISSPA_E_UMBRELLA &&
                  kELj == ISSPA_E_LJ && kEKinAfter == ISSPA_E_KIN_AFTER,
              "energy slots must match the public enum");

int isspa_energies(isspa_engine *e, double *out) {
    if (!e || !out) return ISSPA_ERR_ARG;
    int rc = guard(e);
    if (rc) return rc;
    rc = run_guarded([&] {
        const size_t ne = (size_t)e->n_windows * kECount;
        if (!e->energy) e->energy = e->alloc<double>(ne);
        cudaStream_t s = e->stream;
        ck(cudaStreamSynchronize(s));
        ck(cudaMemsetAsync(e->facc, 0, 3 * sizeof(unsigned long long) * e->n_atoms, s));
        ck(cudaMemsetAsync(e->energy, 0, sizeof(double) * ne, s));
        // the forces of the current step, in the reference order
        launch_bonded(e->bonded_args(1, 1, 1), s);
        e->enqueue_isspa(s);
        e->enqueue_nonbond(s);
        launch_umbrella(e->umbrella_args(), s);
        // energies of the same configuration, and the kick the forces give
        launch_nonbond_energy(e->nonbond_args(), e->energy, s);
        launch_bonded_energy(e->bonded_args(1, 1, 1), e->energy, s);
        launch_state_energy(e->state_energy_args(), e->energy, s);
        ck(cudaGetLastError());
        ck(cudaMemcpyAsync(out, e->energy, sizeof(double) * ne, cudaMemcpyDeviceToHost, s));
        ck(cudaMemsetAsync(e->facc, 0, 3 * sizeof(unsigned long long) * e->n_atoms, s));
        ck(cudaStreamSynchronize(s));
    });
    return rc;
}

int isspa_autotune(isspa_engine *e, int reps, int shape[ISSPA_SHAPE_COUNT]) {
    int rc = guard(e);
    if (rc) return rc;
    if (reps <= 0) reps = 3;
    rc = run_guarded([&] {
        auto time_it = [&](auto &&launch) {
            launch();  // warm-up
            ck(cudaEventRecord(e->ev_a, e->stream));
            for (int r = 0; r < reps; ++r) launch();
            ck(cudaEventRecord(e->ev_b, e->stream));
            ck(cudaEventSynchronize(e->ev_b));
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, e->ev_a, e->ev_b));
            return ms / reps;
        };
        // field pass: every atom-loop split, per-pair and warp-voted loops,
        // atom rounds staged by plain loads and by bulk copies (TMA)
        float best = 1e30f;
        int bestS = e->field_split, bestV = e->field_vote, bestTma = e->field_tma;
        for (int T : {0, 1})
            for (int V : {0, 1})
                for (int S : {1, 2, 4, 8, 16}) {
                    e->set_field_split(S);
                    e->field_vote = V;
                    e->field_tma = T;
                    const float ms = time_it([&] { launch_field(e->field_args(), S, false, e->stream); });
                    if (ms < best) {
                        best = ms;
                        bestS = S;
                        bestV = V;
                        bestTma = T;
                    }
                }
        e->set_field_split(bestS);
        e->field_vote = bestV;
        e->field_tma = bestTma;
        launch_field(e->field_args(), bestS, false, e->stream);
        // force pass: for 1 and 2 atoms per thread, the chunk lengths that fill
        // 1..12 whole waves of that kernel's resident blocks, and powers of two
        long long maxP = 0;
        for (const WinDev &d : e->win_h) maxP = std::max(maxP, (long long)d.n_atoms * e->n_mc);
        best = 1e30f;
        int bestC = e->force_chunk, bestT = e->force_tail, bestA = e->force_apt;
        for (int apt : {1, 2}) {
            e->force_apt = apt;
            const long long slots = (long long)e->n_sms * std::max(1, force_blocks_per_sm(apt));
            std::vector<int> cands = {e->default_force_chunk()};
            for (int k = 1; k <= 12; ++k) {
                long long lo = 32, hi = std::max<long long>(32, std::min<long long>(8192, maxP));
                while (lo < hi) {  // smallest C with items <= k * slots
                    const long long mid = (lo + hi) / 2;
                    if (e->force_items_for(mid) <= k * slots) hi = mid;
                    else lo = mid + 1;
                }
                cands.push_back((int)lo);
            }
            for (int c : {128, 256, 512, 1024, 2048, 4096})
                if (c <= std::max<long long>(128, maxP)) cands.push_back(c);
            std::sort(cands.begin(), cands.end());
            cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
            // (long chunk, short tail chunk) pairs: long items first, then about
            // two waves of short ones
            std::vector<std::pair<int, int>> pairs;
            for (int c : cands) pairs.push_back({c, 0});
            // (8-point tails: a system of a few dozen atoms has fewer points than
            // one wave of 16-point items, and its step waits on the longest
            // thread's chain of points; 4-point tails timed faster alone but
            // slower inside the step)
            for (int c : {64, 128, 256, 512, 1024})
                for (int t : {8, 16, 32, 64})
                    if (t < c && c <= std::max<long long>(128, maxP)) pairs.push_back({c, t});
            for (const auto &ct : pairs) {
                e->set_force_chunk(ct.first, ct.second);
                const float ms = time_it([&] { launch_force(e->force_args(), e->stream); });
                if (ms < best) {
                    best = ms;
                    bestC = ct.first;
                    bestT = ct.second;
                    bestA = apt;
                }
            }
        }
        e->force_apt = bestA;
        e->set_force_chunk(bestC, bestT);
        // the voted force loop (one atom per thread) on the chosen work list
        e->force_vote = 0;
        if (bestA == 1) {
            const float plain = time_it([&] { launch_force(e->force_args(), e->stream); });
            e->force_vote = 1;
            const float voted = time_it([&] { launch_force(e->force_args(), e->stream); });
            e->force_vote = voted < plain ? 1 : 0;
        }
        // nonbond pass: partner stretches per item (results do not move)
        if (e->opt.nonbond_terms && e->n_nb_items > 0 && !e->cutoff) {
            int maxN = 0;
            for (const WinDev &d : e->win_h) maxN = std::max(maxN, d.n_atoms);
            float bestn = 1e30f;
            int bestJ = e->nb_chunk;
            for (int J : {128, 256, 384, 512, 768, 1024, 2048, 4096}) {
                if (J > 128 && J >= maxN + 128) break;
                e->set_nonbond_chunk(J);
                const float ms = time_it([&] { launch_nonbond(e->nonbond_args(), e->stream); });
                if (ms < bestn) {
                    bestn = ms;
                    bestJ = J;
                }
            }
            e->set_nonbond_chunk(bestJ);
        }
        // step mode (the choices the options leave open): integrator,
        // programmatic launches, fused field + force launch, force items on
        // stamped field tiles, timed as single-step graph replays; positions,
        // velocities and the step counter are restored afterwards
        ck(cudaMemsetAsync(e->facc, 0, 3 * sizeof(unsigned long long) * e->n_atoms, e->stream));
        const bool try_fused = e->opt.isspa_fused == 0 && e->fused_applies() &&
                               e->max_window_atoms() <= isspa_engine::kFusedMaxAtoms;
        const bool try_overlap = e->opt.force_overlap == 0 && e->opt.isspa_terms && e->n_force_items > 0;
        if ((e->opt.integrator == 0 || e->opt.step_pdl == 0 || try_fused || try_overlap) && e->n_atoms > 0) {
            std::vector<float4> p0(e->n_atoms), v0(e->n_atoms);
            uint32_t st0 = 0;
            ck(cudaMemcpyAsync(p0.data(), e->pos, sizeof(float4) * e->n_atoms, cudaMemcpyDeviceToHost, e->stream));
            ck(cudaMemcpyAsync(v0.data(), e->vel, sizeof(float4) * e->n_atoms, cudaMemcpyDeviceToHost, e->stream));
            ck(cudaMemcpyAsync(&st0, e->d_step, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream));
            ck(cudaStreamSynchronize(e->stream));
            // candidates: the integrators (1, 2, 3) the options leave open, each
            // with and without programmatic launches of the step chain; the
            // separate passes with and without force items starting on stamped
            // field tiles, and, for small windows, the fused field + force
            // launch at field splits 4, 8 and 16 (its best split need not be the
            // field pass's; none of these in the single-kernel step); three
            // interleaved rounds, the minimum per candidate: they differ by a
            // few per cent where they differ
            struct Cand {
                int m, pdl, fused, split, ov;  // split 0: the field pass's tuned split
            };
            std::vector<Cand> cand;
            const int fixed_fused = e->isspa_fused;
            const int fixed_ov = e->force_overlap;
            const int S0 = e->field_split;
            for (int m : {1, 2, 3}) {
                if (e->opt.integrator != 0 && m != e->integrator) continue;
                if (m == 3 && !e->step_kernel_ok()) continue;
                for (int pdl : {0, 1})
                    for (int fu : {0, 1}) {
                        if (m == 3 && (pdl || fu)) continue;
                        if (e->opt.step_pdl != 0 && m != 3 && pdl != (e->opt.step_pdl == 1 ? 1 : 0)) continue;
                        if (m != 3 && (try_fused ? false : fu != fixed_fused)) continue;
                        size_t added = 0;
                        if (fu && e->fused_applies())
                            for (int S : {4, 8, 16})
                                if (field_force_fusable(S)) {
                                    cand.push_back({m, pdl, 1, S, 0});
                                    ++added;
                                }
                        if (added) continue;
                        // the separate passes (also a fused choice with no fusable split)
                        for (int ov : {0, 1}) {
                            if (m == 3 && ov) continue;
                            if (m != 3 && (try_overlap ? false : ov != fixed_ov)) continue;
                            cand.push_back({m, pdl, fu, 0, ov});
                        }
                    }
            }
            // the field split first (leaving the single-kernel step restores the
            // split it replaced), then the integrator
            auto apply = [&](const Cand &c) {
                e->set_integrator(1);
                const int S = c.split ? c.split : S0;
                if (e->field_split != S) e->set_field_split(S);
                e->set_integrator(c.m);
                e->step_pdl = c.pdl;
                e->isspa_fused = c.fused;
                e->force_overlap = c.ov;
            };
            std::vector<float> t(cand.size(), 1e30f);
            int rounds = 3;
            for (int round = 0; round < rounds; ++round)
                for (size_t c = 0; c < cand.size(); ++c) {
                    apply(cand[c]);
                    e->invalidate_graphs();
                    cudaGraphExec_t g = e->capture(1);
                    auto one = [&] { ck(cudaGraphLaunch(g, e->stream)); };
                    const float first = time_it(one);
                    if (first > 2.0f) rounds = 1;  // long steps: one round is enough
                    const int saved = reps;
                    reps = first > 2.0f ? saved : std::max(saved, 50);
                    t[c] = std::min(t[c], time_it(one));
                    reps = saved;
                    cudaGraphExecDestroy(g);
                }
            size_t best = 0;
            for (size_t c = 1; c < cand.size(); ++c)
                if (t[c] < t[best]) best = c;
            apply(cand[best]);
            ck(cudaMemcpyAsync(e->pos, p0.data(), sizeof(float4) * e->n_atoms, cudaMemcpyHostToDevice, e->stream));
            ck(cudaMemcpyAsync(e->vel, v0.data(), sizeof(float4) * e->n_atoms, cudaMemcpyHostToDevice, e->stream));
            ck(cudaMemcpyAsync(e->d_step, &st0, sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
            ck(cudaMemsetAsync(e->facc, 0, 3 * sizeof(unsigned long long) * e->n_atoms, e->stream));
        }
        ck(cudaStreamSynchronize(e->stream));
        e->invalidate_graphs();
    });
    if (rc) return rc;
    return shape ? isspa_engine_shapes(e, shape) : ISSPA_OK;
}

int isspa_zero_forces(isspa_engine *e) {
    return timed_call(e, nullptr, [&] {
        ck(cudaMemsetAsync(e->facc, 0, 3 * sizeof(unsigned long long) * e->n_atoms, e->stream));
    });
}

int bond_force_cuda(isspa_engine *e, float *ms) {
    return timed_call(e, ms, [&] { launch_bonded(e->bonded_args(1, 0, 0), e->stream); });
}
int angle_force_cuda(isspa_engine *e, float *ms) {
    return timed_call(e, ms, [&] { launch_bonded(e->bonded_args(0, 1, 0), e->stream); });
}
int dih_force_cuda(isspa_engine *e, float *ms) {
    return timed_call(e, ms, [&] { launch_bonded(e->bonded_args(0, 0, 1), e->stream); });
}
int isspa_force_cuda(isspa_engine *e, float *ms) {
    return timed_call(e, ms, [&] { e->enqueue_isspa(e->stream); });
}
int nonbond_force_cuda(isspa_engine *e, float *ms) {
    return timed_call(e, ms, [&] { e->enqueue_nonbond(e->stream); });
}
int us_force_cuda(isspa_engine *e, float *ms) {
    return timed_call(e, ms, [&] { launch_umbrella(e->umbrella_args(), e->stream); });
}
int leapfrog_cuda(isspa_engine *e, float *ms) {
    return timed_call(e, ms, [&] { launch_leapfrog(e->leapfrog_args(), e->stream); });
}

int isspa_step(isspa_engine *e, int nsteps) {
    if (nsteps < 0) return ISSPA_ERR_ARG;
    return timed_call(e, nullptr, [&] { e->run_steps(nsteps); });
}

int isspa_time_steps(isspa_engine *e, int nsteps, size_t flush_bytes, double *ms_total) {
    if (nsteps <= 0 || !ms_total) return ISSPA_ERR_ARG;
    int rc = guard(e);
    if (rc) return rc;
    return run_guarded([&] {
        if (flush_bytes && flush_bytes != e->flush_bytes) {
            if (e->flush) {
                cudaFree(e->flush);
                e->flush = nullptr;
            }
            ck(cudaMalloc(&e->flush, flush_bytes));
            e->flush_bytes = flush_bytes;
        }
        while ((int)e->tev.size() < 2 * nsteps) {
            cudaEvent_t ev;
            ck(cudaEventCreate(&ev));
            e->tev.push_back(ev);
        }
        for (int k = 0; k < nsteps; ++k) {
            if (flush_bytes) ck(cudaMemsetAsync(e->flush, k & 0xff, flush_bytes, e->stream));
            ck(cudaEventRecord(e->tev[2 * k], e->stream));
            e->run_steps(1);
            ck(cudaEventRecord(e->tev[2 * k + 1], e->stream));
        }
        ck(cudaStreamSynchronize(e->stream));
        double tot = 0.0;
        for (int k = 0; k < nsteps; ++k) {
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, e->tev[2 * k], e->tev[2 * k + 1]));
            tot += ms;
        }
        *ms_total = tot;
    });
}

int isspa_time_steps_detailed(isspa_engine *e, int nsteps, size_t flush_bytes, double *ms_total,
                              double *ms_kernels, int *launches) {
    if (nsteps <= 0 || !ms_total || !ms_kernels || !launches) return ISSPA_ERR_ARG;
    int rc = guard(e);
    if (rc) return rc;
    return run_guarded([&] {
        if (flush_bytes && flush_bytes != e->flush_bytes) {
            if (e->flush) {
                cudaFree(e->flush);
                e->flush = nullptr;
            }
            ck(cudaMalloc(&e->flush, flush_bytes));
            e->flush_bytes = flush_bytes;
        }
        if (!e->kev[0])
            for (auto &ev : e->kev) ck(cudaEventCreate(&ev));
        while (e->tev.size() < 2) {
            cudaEvent_t ev;
            ck(cudaEventCreate(&ev));
            e->tev.push_back(ev);
        }
        if (!e->graph_timed) e->graph_timed = e->capture(1, true);
        double tot = 0.0, kt[ISSPA_K_COUNT] = {0};
        int kl[ISSPA_K_COUNT] = {0};
        for (int s = 0; s < nsteps; ++s) {
            if (flush_bytes) ck(cudaMemsetAsync(e->flush, s & 0xff, flush_bytes, e->stream));
            ck(cudaEventRecord(e->tev[0], e->stream));
            ck(cudaGraphLaunch(e->graph_timed, e->stream));
            ck(cudaEventRecord(e->tev[1], e->stream));
            ck(cudaStreamSynchronize(e->stream));
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, e->tev[0], e->tev[1]));
            tot += ms;
            for (int k = 0; k < ISSPA_K_COUNT; ++k) {
                if (!e->launches(k)) continue;
                ck(cudaEventElapsedTime(&ms, e->kev[2 * k], e->kev[2 * k + 1]));
                kt[k] += ms;
                kl[k] += 1;
            }
        }
        *ms_total = tot;
        for (int k = 0; k < ISSPA_K_COUNT; ++k) {
            ms_kernels[k] = kt[k];
            launches[k] = kl[k];
        }
    });
}

int isspa_host_alloc(size_t bytes, void **out) {
    if (!out || !bytes) return ISSPA_ERR_ARG;
    if (cudaHostAlloc(out, bytes, cudaHostAllocPortable | cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return ISSPA_ERR_NOMEM;
    }
    void *dev = nullptr;
    if (cudaHostGetDevicePointer(&dev, *out, 0) == cudaSuccess && dev) {
        std::lock_guard<std::mutex> lock(g_host_mu);
        g_host_bufs[reinterpret_cast<uintptr_t>(*out)] = {bytes, reinterpret_cast<uintptr_t>(dev)};
    } else {
        cudaGetLastError();  // not mapped: isspa_step_host copies it instead
    }
    return ISSPA_OK;
}

void isspa_host_free(void *p) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lock(g_host_mu);
        g_host_bufs.erase(reinterpret_cast<uintptr_t>(p));
    }
    cudaFreeHost(p);
}

int isspa_synchronize(isspa_engine *e) {
    int rc = guard(e);
    if (rc) return rc;
    if (cudaStreamSynchronize(e->stream) != cudaSuccess) {
        cudaGetLastError();
        return ISSPA_ERR_CUDA;
    }
    return isspa_device_status(e, 0);
}

int isspa_device_status(isspa_engine *e, int reset) {
    int rc = guard(e);
    if (rc) return rc;
    // the engine's streams are non-blocking: order the read (and the reset)
    // after the kernels already queued on them
    int st = 0;
    if (cudaStreamSynchronize(e->stream) != cudaSuccess ||
        cudaMemcpyAsync(&st, e->status, sizeof(int), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
        cudaStreamSynchronize(e->stream) != cudaSuccess) {
        cudaGetLastError();
        return ISSPA_ERR_CUDA;
    }
    // a grid barrier that gave up leaves its words mid-count: reset them with the status
    if (reset && (cudaMemsetAsync(e->status, 0, sizeof(int), e->stream) != cudaSuccess ||
                  ((st & kStatusTimeout) && cudaMemsetAsync(e->bar, 0, 2 * sizeof(unsigned int), e->stream) != cudaSuccess) ||
                  cudaStreamSynchronize(e->stream) != cudaSuccess)) {
        cudaGetLastError();
        return ISSPA_ERR_CUDA;
    }
    if (st & kStatusTimeout) return ISSPA_ERR_TIMEOUT;
    if (st & kStatusNonFinite) return ISSPA_ERR_NONFINITE;
    if (st & kStatusOverflow) return ISSPA_ERR_OVERFLOW;
    if (st & kStatusBounds) return ISSPA_ERR_BOUNDS;
    if (st & kStatusListFull) return ISSPA_ERR_LIST_FULL;
    return ISSPA_OK;
}

int isspa_nonbond_list_stats(isspa_engine *e, int *builds, int *fullest_row) {
    if (!e || !builds || !fullest_row) return ISSPA_ERR_ARG;
    int rc = guard(e);
    if (rc) return rc;
    if (!e->cutoff) return ISSPA_ERR_STATE;
    int st[2] = {0, 0};
    rc = run_guarded([&] {
        ck(cudaStreamSynchronize(e->stream));
        ck(cudaMemcpyAsync(st, e->nbl_stats, sizeof st, cudaMemcpyDeviceToHost, e->stream));
        ck(cudaStreamSynchronize(e->stream));
    });
    if (rc) return rc;
    *builds = st[0];
    *fullest_row = st[1];
    return ISSPA_OK;
}

int isspa_debug_stall_barrier(isspa_engine *e) {
    int rc = guard(e);
    if (rc) return rc;
    return run_guarded([&] {
        // an arrival count no grid reaches: every block waits out its limit
        const unsigned int words[2] = {0x80000000u, 0u};
        ck(cudaMemcpyAsync(e->bar, words, sizeof words, cudaMemcpyHostToDevice, e->stream));
        ck(cudaStreamSynchronize(e->stream));
    });
}

static int copy_state(isspa_engine *e, void *dst, const void *src, size_t bytes, cudaMemcpyKind k) {
    int rc = guard(e);
    if (rc) return rc;
    return run_guarded([&] {
        ck(cudaMemcpyAsync(dst, src, bytes, k, e->stream));
        ck(cudaStreamSynchronize(e->stream));
    });
}

int isspa_set_positions(isspa_engine *e, const float *p, int n) {
    if (!e || !p || n != e->n_atoms) return ISSPA_ERR_ARG;
    return copy_state(e, e->pos, p, sizeof(float4) * n, cudaMemcpyHostToDevice);
}
int isspa_get_positions(isspa_engine *e, float *p, int n) {
    if (!e || !p || n != e->n_atoms) return ISSPA_ERR_ARG;
    return copy_state(e, p, e->pos, sizeof(float4) * n, cudaMemcpyDeviceToHost);
}
int isspa_set_velocities(isspa_engine *e, const float *p, int n) {
    if (!e || !p || n != e->n_atoms) return ISSPA_ERR_ARG;
    return copy_state(e, e->vel, p, sizeof(float4) * n, cudaMemcpyHostToDevice);
}
int isspa_get_velocities(isspa_engine *e, float *p, int n) {
    if (!e || !p || n != e->n_atoms) return ISSPA_ERR_ARG;
    return copy_state(e, p, e->vel, sizeof(float4) * n, cudaMemcpyDeviceToHost);
}

int isspa_get_forces(isspa_engine *e, float *f4, int n) {
    if (!e || !f4 || n != e->n_atoms) return ISSPA_ERR_ARG;
    std::vector<long long> acc(3 * (size_t)n);
    int rc = copy_state(e, acc.data(), e->facc, sizeof(long long) * 3 * n, cudaMemcpyDeviceToHost);
    if (rc) return rc;
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) f4[4 * i + k] = (float)((double)acc[3 * i + k] * kFixInv);
        f4[4 * i + 3] = 0.f;
    }
    return ISSPA_OK;
}

int isspa_set_step(isspa_engine *e, uint32_t step) {
    if (!e) return ISSPA_ERR_ARG;
    return copy_state(e, e->d_step, &step, sizeof step, cudaMemcpyHostToDevice);
}
int isspa_get_step(isspa_engine *e, uint32_t *step) {
    if (!e || !step) return ISSPA_ERR_ARG;
    return copy_state(e, step, e->d_step, sizeof *step, cudaMemcpyDeviceToHost);
}

int isspa_get_us_com(isspa_engine *e, double *com, double *cv) {
    if (!e) return ISSPA_ERR_ARG;
    int rc = ISSPA_OK;
    if (com) rc = copy_state(e, com, e->com, sizeof(double) * 6 * e->n_windows, cudaMemcpyDeviceToHost);
    if (!rc && cv) rc = copy_state(e, cv, e->cv, sizeof(double) * e->n_windows, cudaMemcpyDeviceToHost);
    return rc;
}

int isspa_step_host(isspa_engine *e, const float *pin, const float *vin, float *pout, float *vout, float *fout) {
    int rc = guard(e);
    if (rc) return rc;
    const size_t b = sizeof(float4) * e->n_atoms;
    // Buffers that all come from isspa_host_alloc are read and written by two
    // small kernels around the step (the GPU reaches page-locked host memory
    // directly); anything else goes through one copy per buffer.
    const auto *dpin = static_cast<const float4 *>(host_mapped(pin, b));
    const auto *dvin = static_cast<const float4 *>(host_mapped(vin, b));
    auto *dpout = static_cast<float4 *>(host_mapped(pout, b));
    auto *dvout = static_cast<float4 *>(host_mapped(vout, b));
    auto *dfout = static_cast<float4 *>(host_mapped(fout, b));
    const bool direct = (!pin || dpin) && (!vin || dvin) && (!pout || dpout) && (!vout || dvout) && (!fout || dfout);
    return run_guarded([&] {
        if (direct) {
            const Copy3Args in{{dpin, dvin, nullptr}, {e->pos, e->vel, nullptr}, e->n_atoms};
            const Copy3Args out{{pout ? e->pos : nullptr, vout ? e->vel : nullptr, fout ? e->force_out : nullptr},
                                {dpout, dvout, dfout}, e->n_atoms};
            const bool has_in = pin || vin, has_out = pout || vout || fout;
            if (e->opt.use_graph) {
                const void *key[5] = {dpin, dvin, dpout, dvout, dfout};
                ck(cudaGraphLaunch(e->host_step_graph(key, in, has_in, out, has_out), e->stream));
            } else {
                if (has_in) launch_copy3(in, e->stream);
                e->run_steps(1);
                if (has_out) launch_copy3(out, e->stream);
            }
            ck(cudaGetLastError());
        } else {
            if (pin) ck(cudaMemcpyAsync(e->pos, pin, b, cudaMemcpyHostToDevice, e->stream));
            if (vin) ck(cudaMemcpyAsync(e->vel, vin, b, cudaMemcpyHostToDevice, e->stream));
            e->run_steps(1);
            if (pout) ck(cudaMemcpyAsync(pout, e->pos, b, cudaMemcpyDeviceToHost, e->stream));
            if (vout) ck(cudaMemcpyAsync(vout, e->vel, b, cudaMemcpyDeviceToHost, e->stream));
            if (fout) ck(cudaMemcpyAsync(fout, e->force_out, b, cudaMemcpyDeviceToHost, e->stream));
        }
        ck(cudaStreamSynchronize(e->stream));
    });
}

int isspa_set_mc_points(isspa_engine *e, const float *xyz, long long n) {
    if (!e || !xyz || n != e->n_points) return ISSPA_ERR_ARG;
    int rc = guard(e);
    if (rc) return rc;
    rc = run_guarded([&] {
        if (!e->pts_in) e->pts_in = e->alloc<float>(3 * (size_t)e->n_points);
        ck(cudaMemcpyAsync(e->pts_in, xyz, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, e->stream));
        ck(cudaStreamSynchronize(e->stream));
    });
    if (!rc && !e->inject) {
        e->inject = true;
        e->invalidate_graphs();
    }
    return rc;
}

int isspa_clear_mc_points(isspa_engine *e) {
    if (!e) return ISSPA_ERR_ARG;
    if (e->inject) {
        e->inject = false;
        e->invalidate_graphs();
    }
    return ISSPA_OK;
}

int isspa_get_point_fields(isspa_engine *e, float *xyz, float *w, int *n, float *ef, float *e0f, long long np) {
    if (!e || np != e->n_points) return ISSPA_ERR_ARG;
    int rc = guard(e);
    if (rc) return rc;
    return run_guarded([&] {
        if (!e->raw_e) {
            e->raw_e = e->alloc<float4>(e->n_points);
            e->raw_e0 = e->alloc<float4>(e->n_points);
        }
        launch_field(e->field_args(), e->field_split, true, e->stream);
        ck(cudaGetLastError());
        std::vector<float4> a(e->n_points), b(e->n_points), c(e->n_points);
        ck(cudaMemcpyAsync(a.data(), e->raw_e, sizeof(float4) * np, cudaMemcpyDeviceToHost, e->stream));
        ck(cudaMemcpyAsync(b.data(), e->raw_e0, sizeof(float4) * np, cudaMemcpyDeviceToHost, e->stream));
        ck(cudaMemcpyAsync(c.data(), e->pts.q0, sizeof(float4) * np, cudaMemcpyDeviceToHost, e->stream));
        ck(cudaStreamSynchronize(e->stream));
        for (long long p = 0; p < np; ++p) {
            if (xyz) { xyz[3 * p] = c[p].x; xyz[3 * p + 1] = c[p].y; xyz[3 * p + 2] = c[p].z; }
            if (w) w[p] = a[p].w;
            if (n) n[p] = (int)b[p].w;
            if (ef) { ef[3 * p] = a[p].x; ef[3 * p + 1] = a[p].y; ef[3 * p + 2] = a[p].z; }
            if (e0f) { e0f[3 * p] = b[p].x; e0f[3 * p + 1] = b[p].y; e0f[3 * p + 2] = b[p].z; }
        }
    });
}

int isspa_neighbor_list(isspa_engine *e, float rnn, int max_per_atom, int *rows, int *counts) {
    if (!e || !rows || !counts || max_per_atom <= 0 || !(rnn > 0.f)) return ISSPA_ERR_ARG;
    int rc = guard(e);
    if (rc) return rc;
    const WinDev &d = e->win_h[0];
    int *d_rows = nullptr, *d_counts = nullptr;
    // temporary buffers, freed on return, counted against the engine's cap
    const size_t tmp = sizeof(int) * ((size_t)d.n_atoms * max_per_atom + d.n_atoms);
    if (e->opt.mem_cap && e->allocated + tmp > e->opt.mem_cap) return ISSPA_ERR_NOMEM;
    rc = run_guarded([&] {
        ck(cudaMalloc(&d_rows, sizeof(int) * (size_t)d.n_atoms * max_per_atom));
        ck(cudaMalloc(&d_counts, sizeof(int) * d.n_atoms));
        ck(cudaMemsetAsync(d_rows, 0xff, sizeof(int) * (size_t)d.n_atoms * max_per_atom, e->stream));
        ListArgs a{};
        a.pos = e->pos;
        a.excl_start = e->excl_start;
        a.excl = e->excl;
        a.atom_off = d.atom_off;
        a.n_atoms = d.n_atoms;
        a.box = d.box;
        a.hbox = d.hbox;
        a.rnn2 = rnn * rnn;
        a.max_per_atom = max_per_atom;
        a.rows = d_rows;
        a.counts = d_counts;
        launch_neighbor_list(a, e->stream);
        ck(cudaGetLastError());
        ck(cudaMemcpyAsync(rows, d_rows, sizeof(int) * (size_t)d.n_atoms * max_per_atom, cudaMemcpyDeviceToHost, e->stream));
        ck(cudaMemcpyAsync(counts, d_counts, sizeof(int) * d.n_atoms, cudaMemcpyDeviceToHost, e->stream));
        ck(cudaStreamSynchronize(e->stream));
    });
    if (d_rows) cudaFree(d_rows);
    if (d_counts) cudaFree(d_counts);
    return rc;
}

int isspa_cell_list(isspa_engine *e, float rc_len, const int ncell[3], int *cell) {
    if (!e || !ncell || !cell || !(rc_len > 0.f)) return ISSPA_ERR_ARG;
    int rc = guard(e);
    if (rc) return rc;
    const WinDev &d = e->win_h[0];
    int *d_cell = nullptr;
    if (e->opt.mem_cap && e->allocated + sizeof(int) * (size_t)d.n_atoms > e->opt.mem_cap) return ISSPA_ERR_NOMEM;
    rc = run_guarded([&] {
        ck(cudaMalloc(&d_cell, sizeof(int) * d.n_atoms));
        launch_cell_index(e->pos, d.atom_off, d.n_atoms, rc_len, make_int3(ncell[0], ncell[1], ncell[2]), d_cell,
                          e->stream);
        ck(cudaGetLastError());
        ck(cudaMemcpyAsync(cell, d_cell, sizeof(int) * d.n_atoms, cudaMemcpyDeviceToHost, e->stream));
        ck(cudaStreamSynchronize(e->stream));
    });
    if (d_cell) cudaFree(d_cell);
    return rc;
}

int isspa_measure_fp32_peak(double *tflops) {
    if (!tflops) return ISSPA_ERR_ARG;
    double v = measure_fp32_peak_tflops();
    if (v <= 0) return ISSPA_ERR_CUDA;
    *tflops = v;
    return ISSPA_OK;
}

}  // extern "C"
