// k_noalloc.cu -- the IS-SPA force pass for callers that cannot allocate.
//
// Some callers may not call cudaMalloc at all: a host framework that owns every
// device byte through its own pool, a process whose device memory is budgeted
// before it starts, or a time-critical loop that must not take the allocator's
// locks.  isspa_force_noalloc runs the same field and force kernels as the
// engine, but every intermediate array (packed tables, work lists, per-point
// records, fixed-point force accumulator, status word) lives in one file-scope
// device buffer of fixed size.  Inputs and outputs are the caller's device
// arrays.
//
// The buffer is a static __device__ array: every GPU that loads this library
// holds it until the process exits.  Host code cannot use the array's name as a
// device address, so the first call on each device looks the address up with
// cudaGetSymbolAddress (that first call should come before any stream capture)
// and caches it.  All calls share the buffer and it keeps the last call's
// contents; everything that must start at zero is cleared on each call, and
// calls that overlap on the GPU race with each other.
//
// Nothing is copied from host memory: the work lists are pure arithmetic of the
// system's sizes and are written into the buffer by the set-up kernel, so a
// call only enqueues two memsets and four kernels on the caller's stream.
#include <algorithm>
#include <cmath>
#include <mutex>

#include <cuda_runtime.h>

#include "isspa_gb300.h"
#include "kernels.h"

namespace isspa {
namespace {

static_assert(ISSPA_NOALLOC_STATUS_OVERFLOW == kStatusOverflow && ISSPA_NOALLOC_STATUS_NONFINITE == kStatusNonFinite &&
                  ISSPA_NOALLOC_STATUS_BOUNDS == kStatusBounds,
              "status bits of the header and the kernels differ");

static __device__ __align__(256) unsigned char g_noalloc_scratch[ISSPA_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};

// Device address of the scratch buffer and SM count of the current device
// (looked up once per device).
int scratch_address(void **out, int *sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return ISSPA_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        int n = 0;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            return ISSPA_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
        g_sms[dev] = n;
    }
    *out = g_scratch_addr[dev];
    *sms = g_sms[dev];
    return ISSPA_OK;
}

struct Layout {
    size_t off = 0;
    size_t take(size_t bytes) {
        const size_t at = off;
        off = (off + bytes + 255) & ~size_t(255);
        return at;
    }
};

// Sizes of one call's work lists (the engine's list shapes for one window).
struct Plan {
    int n_atoms, tp;              // atoms, MC points per field tile
    long long P, C;               // MC points, points per force chunk
    long long n_tiles, n_chunks, atiles, n_items;
};

struct PrepArgs {
    isspa_noalloc_inputs in;
    Plan plan;
    WinDev *win;
    int4 *tiles, *items;
    int2 *chunks;
    float4 *gtab;
    float2 *ftab;
    float *vtot;
    int2 *atype;
    uint32_t *step;
    int *status;                  // cleared before this kernel runs
};

// Writes everything the field and force kernels read besides the caller's
// arrays: the window record, the field tiles, the force chunks and items
// (chunk-major: co-running blocks read one chunk's point records and add into
// different atom tiles' accumulators), the packed tables with the engine's
// flat-row semantics (a bin's upper neighbour may be the next type's first
// entry; past the last type it reads 0), the per-atom type pairs, vtot
// (isspa_class.cpp:41) and the step key.  An IS-SPA type outside
// [0, n_isspa_types) is replaced by 0 and flags kStatusBounds, so no table is
// read past its end.
__global__ void noalloc_prepare(PrepArgs a) {
    const isspa_noalloc_inputs &in = a.in;
    const Plan &pl = a.plan;
    const int nt = in.n_isspa_types;
    const long long ng = (long long)nt * (in.n_g - 1), nf = (long long)nt * in.n_f;
    const long long gl = (long long)nt * in.n_g, el = (long long)nt * in.n_e;
    long long total = 1;
    for (long long c : {ng, nf, (long long)pl.n_atoms, pl.n_tiles, pl.n_chunks, pl.n_items}) total = c > total ? c : total;
    for (long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x; tid < total;
         tid += (long long)gridDim.x * blockDim.x) {
        if (tid < ng) {
            const long long t = tid / (in.n_g - 1), b = tid % (in.n_g - 1);
            const long long gi = t * in.n_g + b, ei = t * in.n_e + b;
            auto G = [&](long long i) { return i < gl ? in.g_table[i] : 0.0f; };
            auto E = [&](long long i) { return i < el ? in.e_table[i] : 0.0f; };
            a.gtab[tid] = make_float4(G(gi), G(gi + 1), E(ei), E(ei + 1));
        }
        if (tid < nf) a.ftab[tid] = make_float2(in.f_table[tid], tid + 1 < nf ? in.f_table[tid + 1] : 0.0f);
        if (tid < nt) {
            const double r = in.rmax[tid];
            a.vtot[tid] = (float)(4.0 / 3.0 * (double)kPi * r * r * r * 0.0074 / (double)(float)in.n_mc);
        }
        if (tid < pl.n_atoms) {
            int t = in.isspa_type[tid];
            if (t < 0 || t >= nt) {
                atomicOr(a.status, kStatusBounds);
                t = 0;
            }
            a.atype[tid] = make_int2(0, t);
        }
        if (tid < pl.n_tiles)
            a.tiles[tid] = make_int4(0, (int)(tid * pl.tp), (int)min((long long)pl.tp, pl.P - tid * pl.tp), 0);
        if (tid < pl.n_chunks)
            a.chunks[tid] = make_int2((int)(tid * pl.C), (int)min(pl.C, pl.P - tid * pl.C));
        if (tid < pl.n_items) {
            const long long c = tid / pl.atiles, at = tid % pl.atiles;
            a.items[tid] = make_int4(0, (int)(at * 128), (int)min(128LL, pl.n_atoms - at * 128), (int)c);
        }
        if (tid == 0) {
            WinDev w{};
            w.atom_off = 0;
            w.n_atoms = pl.n_atoms;
            w.point_off = 0;
            w.box = in.box;
            w.hbox = 0.5f * in.box;
            *a.win = w;
            *a.step = in.step;
        }
    }
}

// Fixed point to float4 forces; block 0 also reports the call's status word.
__global__ void noalloc_finish(const unsigned long long *facc, int n, float4 *out, const int *status,
                               int *status_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (status_out && i == 0) *status_out = *status;
    if (i >= n) return;
    const unsigned long long *a = facc + 3 * (long long)i;
    out[i] = make_float4((float)((double)(long long)a[0] * kFixInv), (float)((double)(long long)a[1] * kFixInv),
                         (float)((double)(long long)a[2] * kFixInv), 0.0f);
}

}  // namespace
}  // namespace isspa

using namespace isspa;

extern "C" int isspa_force_noalloc(const isspa_noalloc_inputs *in_p, float *force_out, void *stream_p) {
    if (!in_p || !force_out) return ISSPA_ERR_ARG;
    const isspa_noalloc_inputs in = *in_p;
    if (in.n_atoms <= 0 || in.n_mc <= 0 || in.n_isspa_types <= 0 || !in.pos || !in.isspa_type || !in.rmax ||
        !in.g_table || !in.e_table || !in.f_table || in.n_g < 2 || in.n_e < 2 || in.n_f < 2 || !(in.box > 0.f) ||
        !(in.g_dr > 0.f) || !(in.e_dr > 0.f) || !(in.f_dr > 0.f) || in.terms < 0 || in.terms > 7)
        return ISSPA_ERR_ARG;
    const long long P = (long long)in.n_atoms * in.n_mc;
    if (P > INT32_MAX) return ISSPA_ERR_UNSUPPORTED;
    cudaStream_t stream = (cudaStream_t)stream_p;
    void *base = nullptr;
    int sms = 0;
    int rc = scratch_address(&base, &sms);
    if (rc) return rc;

    // launch shapes: field split by wave efficiency, force chunks for >= 2 waves
    auto eff = [](long long u, long long s) {
        if (u <= 0 || s <= 0) return 0.0;
        const double w = (double)u / (double)s;
        return w / std::ceil(w);
    };
    int S = 4;
    double best = -1.0;
    for (int c : {1, 2, 4, 8, 16}) {
        const int tp = field_points_per_block(c);
        const double e = eff((P + tp - 1) / tp, (long long)sms * field_blocks_per_sm(c));
        if (e > best + 0.02) {
            best = e;
            S = c;
        }
    }
    Plan pl{};
    pl.n_atoms = in.n_atoms;
    pl.tp = field_points_per_block(S);
    pl.P = P;
    pl.atiles = (in.n_atoms + 127) / 128;
    const long long fslots = (long long)sms * std::max(1, force_blocks_per_sm(1));
    pl.C = std::max<long long>(64, std::min<long long>(8192, (pl.atiles * P + 2 * fslots - 1) / (2 * fslots)));
    pl.n_tiles = (P + pl.tp - 1) / pl.tp;
    pl.n_chunks = (P + pl.C - 1) / pl.C;
    pl.n_items = pl.atiles * pl.n_chunks;

    // scratch layout
    const int nt = in.n_isspa_types;
    Layout L;
    const size_t o_win = L.take(sizeof(WinDev));
    const size_t o_tiles = L.take(sizeof(int4) * pl.n_tiles);
    const size_t o_items = L.take(sizeof(int4) * pl.n_items);
    const size_t o_chunks = L.take(sizeof(int2) * pl.n_chunks);
    const size_t o_gtab = L.take(sizeof(float4) * (size_t)nt * (in.n_g - 1));
    const size_t o_ftab = L.take(sizeof(float2) * (size_t)nt * in.n_f);
    const size_t o_vtot = L.take(sizeof(float) * nt);
    const size_t o_atype = L.take(sizeof(int2) * in.n_atoms);
    const size_t o_facc = L.take(sizeof(unsigned long long) * 3 * (size_t)in.n_atoms);
    size_t o_q[5];
    for (int k = 0; k < 5; ++k) o_q[k] = L.take(sizeof(float4) * (size_t)P);
    const size_t o_step = L.take(sizeof(uint32_t));
    const size_t o_status = L.take(sizeof(int));
    if (L.off > ISSPA_NOALLOC_SCRATCH_BYTES) return ISSPA_ERR_UNSUPPORTED;
    unsigned char *b = static_cast<unsigned char *>(base);
    int *status = (int *)(b + o_status);

    if (cudaMemsetAsync(status, 0, sizeof(int), stream) != cudaSuccess ||
        cudaMemsetAsync(b + o_facc, 0, sizeof(unsigned long long) * 3 * (size_t)in.n_atoms, stream) != cudaSuccess) {
        cudaGetLastError();
        return ISSPA_ERR_CUDA;
    }
    PrepArgs pa{};
    pa.in = in;
    pa.plan = pl;
    pa.win = (WinDev *)(b + o_win);
    pa.tiles = (int4 *)(b + o_tiles);
    pa.items = (int4 *)(b + o_items);
    pa.chunks = (int2 *)(b + o_chunks);
    pa.gtab = (float4 *)(b + o_gtab);
    pa.ftab = (float2 *)(b + o_ftab);
    pa.vtot = (float *)(b + o_vtot);
    pa.atype = (int2 *)(b + o_atype);
    pa.step = (uint32_t *)(b + o_step);
    pa.status = status;
    const long long prep = std::max({(long long)nt * (in.n_g - 1), (long long)nt * in.n_f, (long long)in.n_atoms,
                                     pl.n_tiles, pl.n_chunks, pl.n_items, 1LL});
    noalloc_prepare<<<(unsigned)std::min<long long>((prep + 255) / 256, 4LL * sms), 256, 0, stream>>>(pa);

    PointsDev pts{(float4 *)(b + o_q[0]), (float4 *)(b + o_q[1]), (float4 *)(b + o_q[2]), (float4 *)(b + o_q[3]),
                  (float4 *)(b + o_q[4])};
    const int terms = in.terms ? in.terms : 7;
    FieldArgs fa{};
    fa.pos = (const float4 *)in.pos;
    fa.atype = pa.atype;
    fa.win = pa.win;
    fa.tiles = pa.tiles;
    fa.n_tiles = (int)pl.n_tiles;
    fa.gtab = pa.gtab;
    fa.rmax = in.rmax;
    fa.n_gbins = in.n_g - 1;
    fa.g_r0 = in.g_r0;
    fa.g_dr = in.g_dr;
    fa.g_inv = 1.0f / in.g_dr;
    fa.e_r0 = in.e_r0;
    fa.e_dr = in.e_dr;
    fa.e_inv = 1.0f / in.e_dr;
    fa.e0 = 3.0f / (4.0f * kPi * kRho * kP0) * (1.0f - 1.0f / kEp);
    fa.n_mc = in.n_mc;
    fa.seed_lo = (uint32_t)in.seed;
    fa.seed_hi = (uint32_t)(in.seed >> 32);
    fa.step_ptr = pa.step;
    fa.pts_in = nullptr;
    fa.out = pts;
    fa.terms = terms;
    fa.status = status;
    launch_field(fa, S, false, stream);

    ForceArgs ka{};
    ka.pos = (const float4 *)in.pos;
    ka.atype = pa.atype;
    ka.win = pa.win;
    ka.items = pa.items;
    ka.chunks = pa.chunks;
    ka.n_items = (int)pl.n_items;
    ka.pts = pts;
    ka.ftab = pa.ftab;
    ka.rmax = in.rmax;
    ka.vtot = pa.vtot;
    ka.n_f = in.n_f;
    ka.f_r0 = in.f_r0;
    ka.f_dr = in.f_dr;
    ka.f_inv = 1.0f / in.f_dr;
    ka.terms = terms;
    ka.atoms_per_thread = 1;
    ka.facc = (unsigned long long *)(b + o_facc);
    ka.status = status;
    launch_force(ka, stream);
    noalloc_finish<<<(in.n_atoms + 127) / 128, 128, 0, stream>>>(ka.facc, in.n_atoms, (float4 *)force_out, status,
                                                                 in.status_out);
    if (cudaGetLastError() != cudaSuccess) return ISSPA_ERR_CUDA;
    return ISSPA_OK;
}
