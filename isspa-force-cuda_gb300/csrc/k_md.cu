// k_md.cu -- pair, bonded, umbrella and integrator kernels for sm_103a.
//
//  nonbond:  all-pairs LJ + Coulomb + IS-SPA long-range dielectric correction
//            (reference src/nonbond_force_cuda.cu:31-174).  One thread per
//            receiving atom, partner atoms streamed through shared memory,
//            exclusions from a per-atom sorted list walked with a cursor (the
//            reference copies the whole list into shared memory per block and
//            fails once it exceeds 48 KB).
//  bonded:   bonds, angles, dihedrals with scaled 1-4 (bond_force_cuda.cu:
//            15-53, angle_force_cuda.cu:12-66, dih_force_cuda.cu:13-136) in one
//            launch over the concatenated term lists.
//  umbrella: one block per restrained window: FP64 centre-of-mass reduction,
//            then the harmonic COM-distance force (us_force_cuda.cu:14-48,
//            whose __syncthreads only orders a single block).
//  leapfrog: consumes and clears the fixed-point force accumulator, Andersen
//            collisions from Philox, leapfrog update and wrap
//            (leapfrog_cuda.cu:33-68).
#include <algorithm>
#include <climits>
#include <cuda_runtime.h>

#include "kernels.h"
#include "md_device.cuh"
#include "philox.h"

namespace isspa {

namespace {

template <bool SMEM_AB, bool ALL>
__global__ void __launch_bounds__(kNbThreads, 8) nonbond_kernel(NonbondArgs a) {
    extern __shared__ float2 s_ab[];
    if (SMEM_AB) stage_ljab(a, s_ab);
    nonbond_item<SMEM_AB, ALL>(a, blockIdx.x, s_ab);
}

__global__ void bonded_kernel(BondedArgs a) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bonded_term(a, idx, FixAdd{a.facc, a.status});
}

__global__ void __launch_bounds__(kUsThreads) umbrella_kernel(UmbrellaArgs a) {
    __shared__ double s_red[6 * kUsThreads];
    __shared__ double s_f[4];
    const int w = a.us_windows[blockIdx.x];
    umbrella_com_block(a, w, s_red, s_f);
    const WinDev W = a.win[w];
    for (int b = threadIdx.x; b < W.n_bias; b += kUsThreads) {
        long long f[3];
        umbrella_entry_fix(a, W, b, s_f, f);
        unsigned long long *acc = a.facc + 3 * (long long)a.bias[W.bias_off + b].x;
        for (int k = 0; k < 3; ++k) atomicAdd(acc + k, (unsigned long long)f[k]);
    }
}

// Every block reads the step counter first; the last block to finish
// advances it (no block waits on another).  A single block advances it after
// its own barrier, without the completion count.
__global__ void leapfrog_kernel(LeapfrogArgs a) {
    pdl_wait();
    pdl_trigger();
    const uint32_t step = *a.step_ptr;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n_atoms) leapfrog_atom(a, i, step, nullptr);
    __syncthreads();
    if (gridDim.x == 1) {
        if (threadIdx.x == 0) {
            *a.step_ptr = step + 1u;
            if (a.ov_epoch) ++*a.ov_epoch;
        }
        return;
    }
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int prev = atomicAdd(a.done_ptr, 1u);
        if (prev == gridDim.x - 1) {
            *a.step_ptr = step + 1u;
            if (a.ov_epoch) ++*a.ov_epoch;
            *a.done_ptr = 0u;
            __threadfence();
        }
    }
}

// The fused integrator: bonded terms, the umbrella restraint and leapfrog in
// one cooperative launch.  Phase 1: blocks take the restrained windows' FP64
// COMs (one block per window, fixed order) and every thread a share of the
// bonded terms (fixed-point atomics, the bonded kernel's term code).  Grid
// barrier.  Phase 2: every atom adds its restraint force from its window's
// COM axis (the umbrella kernel's fixed-point values, no atomics) and is
// integrated; block 0 advances the step counter.  The integer sums are those
// of the separate bonded, umbrella and leapfrog kernels, so the trajectory is
// bit-identical to theirs.
__global__ void __launch_bounds__(kUsThreads) integrator_kernel(IntegratorArgs a) {
    const uint32_t step = *a.lf.step_ptr;
    restraint_coms(a);
    bonded_terms(a.bonded);
    if (!grid_barrier(a.bar, a.lf.status)) return;
    integrate_atoms(a, step);
}

// Neighbour list of one window: one warp per atom, partners scanned in
// ascending order and appended with a warp ballot, so every row comes out
// sorted and identical run to run (the reference appends in atomic order,
// neighborlist_cuda.cu:85-96).
__global__ void neighbor_list_kernel(ListArgs a) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= a.n_atoms) return;
    const int i = a.atom_off + warp;
    const float4 xi = a.pos[i];
    const int ex0 = a.excl_start[i], ex1 = a.excl_start[i + 1];
    int count = 0;
    for (int j0 = 0; j0 < a.n_atoms; j0 += 32) {
        const int jl = j0 + lane;
        bool hit = false;
        if (jl < a.n_atoms && jl != warp) {
            const int j = a.atom_off + jl;
            const float4 xj = a.pos[j];
            const float rx = mimg(xi.x - xj.x, a.box, a.hbox);
            const float ry = mimg(xi.y - xj.y, a.box, a.hbox);
            const float rz = mimg(xi.z - xj.z, a.box, a.hbox);
            hit = dist2f(rx, ry, rz) < a.rnn2;
            if (hit)
                for (int e = ex0; e < ex1; ++e)
                    if (a.excl[e] == j) {
                        hit = false;
                        break;
                    }
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int slot = count + __popc(m & ((1u << lane) - 1u));
            if (slot < a.max_per_atom) a.rows[(long long)warp * a.max_per_atom + slot] = jl;
        }
        count += __popc(m);
    }
    if (lane == 0) a.counts[warp] = count;
}

__global__ void cell_index_kernel(const float4 *pos, int off, int n, float rc, int3 nc, int *cell) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = pos[off + i];
    // cell_list_cuda.cu:27-29
    cell[i] = (int)(x.x / rc) * nc.y * nc.z + (int)(x.y / rc) * nc.z + (int)(x.z / rc);
}

__global__ void fma_peak_kernel(float *out, int iters, float seed) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.999999f, c = 1.0e-7f;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

}  // namespace

int nonbond_block_threads() { return kNbThreads; }

void launch_nonbond(const NonbondArgs &a, cudaStream_t s) {
    if (a.n_items <= 0) return;
    const int nab = a.n_lj_types * a.n_lj_types;
    const bool all = a.terms == 7;
    if (nab <= kNbMaxAB) {
        const size_t sm = sizeof(float2) * (size_t)std::max(nab, 1);
        if (all) nonbond_kernel<true, true><<<a.n_items, kNbThreads, sm, s>>>(a);
        else nonbond_kernel<true, false><<<a.n_items, kNbThreads, sm, s>>>(a);
    } else {
        if (all) nonbond_kernel<false, true><<<a.n_items, kNbThreads, 0, s>>>(a);
        else nonbond_kernel<false, false><<<a.n_items, kNbThreads, 0, s>>>(a);
    }
}

int nonbond_blocks_per_sm(int n_lj_types) {
    int n = 0;
    const int nab = n_lj_types * n_lj_types;
    if (nab <= kNbMaxAB)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, nonbond_kernel<true, true>, kNbThreads,
                                                      sizeof(float2) * (size_t)std::max(nab, 1));
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, nonbond_kernel<false, true>, kNbThreads, 0);
    return n;
}

void launch_bonded(const BondedArgs &a, cudaStream_t s) {
    long long n = (a.do_bonds ? a.n_bonds : 0) + (a.do_angles ? a.n_angles : 0) + (a.do_dihs ? a.n_dihs : 0);
    if (n <= 0) return;
    const int tpb = 128;
    bonded_kernel<<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, s>>>(a);
}

void launch_umbrella(const UmbrellaArgs &a, cudaStream_t s) {
    if (a.n_us_windows > 0) umbrella_kernel<<<a.n_us_windows, kUsThreads, 0, s>>>(a);
}

int integrator_block_threads() { return kUsThreads; }

int integrator_max_blocks() {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, integrator_kernel, kUsThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return sms * per_sm;
}

cudaError_t launch_integrator(const IntegratorArgs &a, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kUsThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, integrator_kernel, a);
}

namespace {
thread_local bool t_chain_pdl = false;
}
bool chain_pdl() { return t_chain_pdl; }
PdlScope::PdlScope(bool on) : prev_(t_chain_pdl) { t_chain_pdl = on; }
PdlScope::~PdlScope() { t_chain_pdl = prev_; }

void launch_leapfrog(const LeapfrogArgs &a, cudaStream_t s) {
    if (a.n_atoms > 0) launch_chain(leapfrog_kernel, (a.n_atoms + 127) / 128, 128, s, a);
}

void launch_neighbor_list(const ListArgs &a, cudaStream_t s) {
    if (a.n_atoms <= 0) return;
    const long long threads = (long long)a.n_atoms * 32;
    neighbor_list_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(a);
}

void launch_cell_index(const float4 *pos, int off, int n, float rc, int3 nc, int *cell, cudaStream_t s) {
    if (n > 0) cell_index_kernel<<<(n + 127) / 128, 128, 0, s>>>(pos, off, n, rc, nc, cell);
}

__global__ void copy3_kernel(Copy3Args a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (a.src[k]) a.dst[k][i] = a.src[k][i];
}

void launch_copy3(const Copy3Args &a, cudaStream_t s) {
    if (a.n > 0) copy3_kernel<<<(a.n + 255) / 256, 256, 0, s>>>(a);
}

double measure_fp32_peak_tflops() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return -1.0;
    const int threads = 256, blocks = sms * 8, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_peak_kernel<<<blocks, threads>>>(out, 64, 1.0f);  // warm-up
    cudaEventRecord(e0);
    fma_peak_kernel<<<blocks, threads>>>(out, iters, 1.0f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
    const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
    return flops / (ms * 1e-3) / 1e12;
}

}  // namespace isspa
