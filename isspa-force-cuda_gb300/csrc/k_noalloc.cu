// k_noalloc.cu -- the IS-SPA force pass for callers that cannot allocate.
//
// Some callers may not call cudaMalloc at all: a host framework that owns every
// device byte through its own pool, a process whose device memory is budgeted
// before it starts, or a time-critical loop that must not take the allocator's
// locks.  isspa_force_noalloc runs the same field and force kernels as the
// engine, but every intermediate array (packed tables, work lists, per-point
// records, fixed-point force accumulator) lives in one file-scope device buffer
// of fixed size.  Inputs and outputs are the caller's device arrays.
//
// The buffer is a static __device__ array: every GPU that loads this library
// holds it until the process exits.  Host code cannot use the array's name as a
// device address, so the first call on each device looks the address up with
// cudaGetSymbolAddress (that call should come before any stream capture) and
// caches it.  All calls share the buffer and it keeps the last call's
// contents; everything that must start at zero is cleared on each call, and
// calls that overlap on the GPU race with each other.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "isspa_gb300.h"
#include "kernels.h"

namespace isspa {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[ISSPA_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch buffer on the current device (looked up once).
int scratch_address(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return ISSPA_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return ISSPA_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
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

// Packs the caller's tables with the engine's flat-row semantics (a bin's
// upper neighbour may be the next type's first entry; past the last type it
// reads 0), the per-atom type pairs, vtot (isspa_class.cpp:41), the step key,
// and clears the status word.
__global__ void noalloc_prepare(isspa_noalloc_inputs in, float4 *gtab, float2 *ftab, float *vtot, int2 *atype,
                                uint32_t *step, int *status) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = in.n_isspa_types;
    const int ng = nt * (in.n_g - 1), nf = nt * in.n_f;
    const long long gl = (long long)nt * in.n_g, el = (long long)nt * in.n_e, fl = (long long)nt * in.n_f;
    auto G = [&](long long i) { return i < gl ? in.g_table[i] : 0.0f; };
    auto E = [&](long long i) { return i < el ? in.e_table[i] : 0.0f; };
    auto F = [&](long long i) { return i < fl ? in.f_table[i] : 0.0f; };
    if (tid < ng) {
        const int t = tid / (in.n_g - 1), b = tid % (in.n_g - 1);
        const long long gi = (long long)t * in.n_g + b, ei = (long long)t * in.n_e + b;
        gtab[tid] = make_float4(G(gi), G(gi + 1), E(ei), E(ei + 1));
    }
    if (tid < nf) ftab[tid] = make_float2(F(tid), F(tid + 1));
    if (tid < nt) {
        const double r = in.rmax[tid];
        vtot[tid] = (float)(4.0 / 3.0 * (double)kPi * r * r * r * 0.0074 / (double)(float)in.n_mc);
    }
    if (tid < in.n_atoms) atype[tid] = make_int2(0, in.isspa_type[tid]);
    if (tid == 0) {
        *step = in.step;
        *status = 0;
    }
}

__global__ void noalloc_finish(const unsigned long long *facc, int n, float4 *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
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
        !(in.g_dr > 0.f) || !(in.e_dr > 0.f) || !(in.f_dr > 0.f))
        return ISSPA_ERR_ARG;
    const long long P = (long long)in.n_atoms * in.n_mc;
    if (P > INT32_MAX) return ISSPA_ERR_UNSUPPORTED;
    cudaStream_t stream = (cudaStream_t)stream_p;
    void *base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;

    // launch shapes: field split by wave efficiency, force chunks for >= 2 waves
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return ISSPA_ERR_CUDA;
    }
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
    const int tp = field_points_per_block(S);
    const long long atiles = (in.n_atoms + 127) / 128;
    const long long fslots = (long long)sms * std::max(1, force_blocks_per_sm(1));
    long long C = std::max<long long>(64, std::min<long long>(8192, (atiles * P + 2 * fslots - 1) / (2 * fslots)));
    const long long n_tiles = (P + tp - 1) / tp, n_chunks = (P + C - 1) / C, n_items = atiles * n_chunks;

    // scratch layout
    const int nt = in.n_isspa_types;
    Layout L;
    const size_t o_win = L.take(sizeof(WinDev));
    const size_t o_tiles = L.take(sizeof(int4) * n_tiles);
    const size_t o_items = L.take(sizeof(int4) * n_items);
    const size_t o_chunks = L.take(sizeof(int2) * n_chunks);
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

    // host-built work lists, copied into the scratch buffer
    WinDev w{};
    w.atom_off = 0;
    w.n_atoms = in.n_atoms;
    w.point_off = 0;
    w.box = in.box;
    w.hbox = 0.5f * in.box;
    std::vector<int4> tiles(n_tiles), items(n_items);
    std::vector<int2> chunks(n_chunks);
    for (long long t = 0; t < n_tiles; ++t)
        tiles[t] = make_int4(0, (int)(t * tp), (int)std::min<long long>(tp, P - t * tp), 0);
    for (long long c = 0; c < n_chunks; ++c) chunks[c] = make_int2((int)(c * C), (int)std::min<long long>(C, P - c * C));
    for (long long a = 0, k = 0; a < atiles; ++a)
        for (long long c = 0; c < n_chunks; ++c, ++k)
            items[k] = make_int4(0, (int)(a * 128), (int)std::min<long long>(128, in.n_atoms - a * 128), (int)c);
    if (cudaMemcpyAsync(b + o_win, &w, sizeof w, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemcpyAsync(b + o_tiles, tiles.data(), sizeof(int4) * n_tiles, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemcpyAsync(b + o_items, items.data(), sizeof(int4) * n_items, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemcpyAsync(b + o_chunks, chunks.data(), sizeof(int2) * n_chunks, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemsetAsync(b + o_facc, 0, sizeof(unsigned long long) * 3 * (size_t)in.n_atoms, stream) != cudaSuccess) {
        cudaGetLastError();
        return ISSPA_ERR_CUDA;
    }
    const long long prep = std::max<long long>({(long long)nt * (in.n_g - 1), (long long)nt * in.n_f, in.n_atoms, 1});
    noalloc_prepare<<<(unsigned)((prep + 255) / 256), 256, 0, stream>>>(
        in, (float4 *)(b + o_gtab), (float2 *)(b + o_ftab), (float *)(b + o_vtot), (int2 *)(b + o_atype),
        (uint32_t *)(b + o_step), (int *)(b + o_status));

    PointsDev pts{(float4 *)(b + o_q[0]), (float4 *)(b + o_q[1]), (float4 *)(b + o_q[2]), (float4 *)(b + o_q[3]),
                  (float4 *)(b + o_q[4])};
    const int terms = in.terms ? in.terms : 7;
    FieldArgs fa{};
    fa.pos = (const float4 *)in.pos;
    fa.atype = (const int2 *)(b + o_atype);
    fa.win = (const WinDev *)(b + o_win);
    fa.tiles = (const int4 *)(b + o_tiles);
    fa.n_tiles = (int)n_tiles;
    fa.gtab = (const float4 *)(b + o_gtab);
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
    fa.step_ptr = (const uint32_t *)(b + o_step);
    fa.pts_in = nullptr;
    fa.out = pts;
    fa.terms = terms;
    fa.status = (int *)(b + o_status);
    launch_field(fa, S, false, stream);

    ForceArgs ka{};
    ka.pos = (const float4 *)in.pos;
    ka.atype = (const int2 *)(b + o_atype);
    ka.win = (const WinDev *)(b + o_win);
    ka.items = (const int4 *)(b + o_items);
    ka.chunks = (const int2 *)(b + o_chunks);
    ka.n_items = (int)n_items;
    ka.pts = pts;
    ka.ftab = (const float2 *)(b + o_ftab);
    ka.rmax = in.rmax;
    ka.vtot = (const float *)(b + o_vtot);
    ka.n_f = in.n_f;
    ka.f_r0 = in.f_r0;
    ka.f_dr = in.f_dr;
    ka.f_inv = 1.0f / in.f_dr;
    ka.terms = terms;
    ka.facc = (unsigned long long *)(b + o_facc);
    ka.status = (int *)(b + o_status);
    launch_force(ka, stream);
    noalloc_finish<<<(in.n_atoms + 127) / 128, 128, 0, stream>>>((const unsigned long long *)(b + o_facc), in.n_atoms,
                                                                 (float4 *)force_out);
    if (cudaGetLastError() != cudaSuccess) return ISSPA_ERR_CUDA;
    return ISSPA_OK;
}
