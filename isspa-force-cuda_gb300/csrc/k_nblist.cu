// k_nblist.cu -- the optional cutoff mode of the nonbond pass: a Verlet
// neighbour list over per-window cell lists, rebuilt on the device.
//
// The reference's live path has no cutoff: its nonbond kernel evaluates every
// pair (nonbond_force_cuda.cu:31-174; the `rCut2` it is handed is unused), and
// its neighbour-list and cell-list kernels (neighborlist_cuda.cu:11-137,
// cell_list_cuda.cu:13-35) are built but never called.  Here a cutoff rc > 0
// truncates all three nonbond terms (LJ, Coulomb, IS-SPA correction) at rc with
// no shift: a pair counts iff its FP32 squared minimum-image distance is below
// rc^2.  Per step:
//   check    every atom's displacement since the last build; any beyond half
//            the skin (or the first step) sets the rebuild flag;
//   bin      (rebuild only) cell of every atom: cells per window edge
//            nc = floor(box / (1.0001 (rc + skin))), or the whole window as
//            one cell when nc < 3;
//   scan     (rebuild only) cell starts, one block;
//   scatter  (rebuild only) atoms into their cells;
//   rows     (rebuild only) per atom, every partner within rc + skin from the
//            27 neighbouring cells (or the whole window), with the exclusion
//            bit from the atom's sorted exclusion list (excluded pairs keep
//            the IS-SPA correction, nonbond_force_cuda.cu:153-162);
//   pairs    per atom, the row's pairs closer than rc.
// A pair within rc now was within rc + skin at the last build, because no atom
// has since moved more than skin / 2, so the pairs evaluated are exactly the
// pairs within rc.  Every pair's force is rounded to the fixed-point grid on
// its own and summed as integers, so the force does not depend on the order of
// a row, on the skin or on when the list was rebuilt.
#include <climits>
#include <cmath>

#include "kernels.h"

namespace isspa {
namespace {

constexpr int kNblThreads = 256;  // 8 warps: one atom per warp in rows / pairs
constexpr unsigned kFull = 0xffffffffu;

// Cell coordinate in [0, nc) of a coordinate wrapped into the box (any finite
// or non-finite x maps into range; non-finite positions are reported by the
// force checks).
__device__ __forceinline__ int cell_coord(float x, float scale, int nc) {
    int c = (int)floorf(x * scale) % nc;
    return c < 0 ? c + nc : c;
}

// j in the sorted exclusion list ex[lo, end)?
__device__ __forceinline__ bool excluded(const int *ex, int lo, int end, int j) {
    int hi = end;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ex[mid] < j) lo = mid + 1;
        else hi = mid;
    }
    return lo < end && ex[lo] == j;
}

__global__ void nbl_check_kernel(NbListArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool move = false;
    if (i < a.n_atoms) {
        const WinDev &W = a.win[a.atom_win[i]];
        const float L = W.box, h = W.hbox;
        const float4 p = a.pos[i], r = a.ref[i];
        const float d2 = dist2f(mimg(p.x - r.x, L, h), mimg(p.y - r.y, L, h), mimg(p.z - r.z, L, h));
        move = !(d2 <= a.half_skin2);  // NaN (before the first build) rebuilds
    }
    if (__any_sync(kFull, move) && (threadIdx.x & 31) == 0) atomicOr(a.flag, 1);
}

__global__ void nbl_bin_kernel(NbListArgs a) {
    if (!*a.flag) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_atoms) return;
    const int4 wc = a.wcell[a.atom_win[i]];  // first cell, cells per edge, scale bits, -
    int c = wc.x;
    if (wc.y > 1) {
        const float4 p = a.pos[i];
        const float sc = __int_as_float(wc.z);
        const int nc = wc.y;
        c += (cell_coord(p.x, sc, nc) * nc + cell_coord(p.y, sc, nc)) * nc + cell_coord(p.z, sc, nc);
    }
    a.cell_of[i] = c;
    atomicAdd(a.cell_count + c, 1);
}

// Exclusive scan of the cell counts into starts (and scatter cursors); the
// counts are cleared for the next build.  One block of 1024 threads.
__global__ void __launch_bounds__(1024) nbl_scan_kernel(NbListArgs a) {
    if (!*a.flag) return;
    __shared__ int s_warp[32];
    __shared__ int s_carry;
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    if (t == 0) {
        s_carry = 0;
        a.stats[0] += 1;  // builds so far
        a.stats[1] = 0;   // fullest row of this build
    }
    for (int base = 0; base < a.n_cells; base += 1024) {
        __syncthreads();
        const int c = base + t;
        const int v = c < a.n_cells ? a.cell_count[c] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int w = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(kFull, w, o);
                if (lane >= o) w += y;
            }
            s_warp[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const int before = s_carry + (wid ? s_warp[wid - 1] : 0) + x - v;
        if (c < a.n_cells) {
            a.cell_start[c] = before;
            a.cell_cursor[c] = before;
            a.cell_count[c] = 0;
        }
        __syncthreads();
        if (t == 1023) s_carry = before + v;
    }
    __syncthreads();
    if (t == 0) a.cell_start[a.n_cells] = s_carry;
}

__global__ void nbl_scatter_kernel(NbListArgs a) {
    if (!*a.flag) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_atoms) return;
    a.cell_atoms[atomicAdd(a.cell_cursor + a.cell_of[i], 1)] = i;
}

// One warp per atom: every partner within rc + skin, compacted by ballot.
// Entries are j | (excluded << 31); a row holds at most row_cap of them (the
// count beyond that is kept and reported).  With rows == nullptr only the
// counts are taken (sizing the rows at engine creation).
__global__ void nbl_rows_kernel(NbListArgs a) {
    if (!*a.flag) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= a.n_atoms) return;  // warp-uniform
    const WinDev &W = a.win[a.atom_win[i]];
    const int4 wc = a.wcell[a.atom_win[i]];
    const float L = W.box, h = W.hbox;
    const float4 xi = a.pos[i];
    const int e0 = a.excl_start[i], e1 = a.excl_start[i + 1];
    int *row = a.rows ? a.rows + (long long)i * a.row_cap : nullptr;
    int count = 0;
    auto take = [&](int j) {  // this lane's candidate, or -1
        bool hit = false, ex = false;
        if (j >= 0 && j != i) {
            const float4 xj = a.pos[j];
            const float d2 = dist2f(mimg(xi.x - xj.x, L, h), mimg(xi.y - xj.y, L, h), mimg(xi.z - xj.z, L, h));
            hit = d2 < a.list2;
            if (hit) ex = excluded(a.excl, e0, e1, j);
        }
        const unsigned m = __ballot_sync(kFull, hit);
        if (hit && row) {
            const int slot = count + __popc(m & ((1u << lane) - 1u));
            if (slot < a.row_cap) row[slot] = j | (ex ? INT_MIN : 0);
        }
        count += __popc(m);
    };
    if (wc.y <= 1) {
        const int j1 = W.atom_off + W.n_atoms;
        for (int j0 = W.atom_off; j0 < j1; j0 += 32) take(j0 + lane < j1 ? j0 + lane : -1);
    } else {
        const int nc = wc.y;
        const int r = a.cell_of[i] - wc.x;
        const int cz = r % nc, cy = (r / nc) % nc, cx = r / (nc * nc);
        for (int dx = nc - 1; dx <= nc + 1; ++dx)
            for (int dy = nc - 1; dy <= nc + 1; ++dy)
                for (int dz = nc - 1; dz <= nc + 1; ++dz) {
                    const int c = wc.x + (((cx + dx) % nc) * nc + (cy + dy) % nc) * nc + (cz + dz) % nc;
                    const int k1 = a.cell_start[c + 1];
                    for (int k0 = a.cell_start[c]; k0 < k1; k0 += 32)
                        take(k0 + lane < k1 ? a.cell_atoms[k0 + lane] : -1);
                }
    }
    if (lane == 0) {
        a.row_n[i] = count;
        a.ref[i] = xi;
        atomicMax(a.stats + 1, count);
        if (row && count > a.row_cap) atomicOr(a.status, kStatusListFull);
    }
}

// One warp per atom over its row: the pairs closer than rc, each force rounded
// to the fixed-point grid on its own (order-free integer sums).  Pair forces
// as the all-pairs kernel: LJ r^-6 (12A r^-6 - 6B) / r^2 (nonbond_force_cuda.cu:
// 131-132), Coulomb q q / r^3 (:136), IS-SPA correction with the partner's
// rmax (:141-147), excluded pairs the correction only (:153-162).
template <bool ALL>
__global__ void __launch_bounds__(kNblThreads) nbl_pairs_kernel(NbListArgs a) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.flag = 0;  // read by no block of this kernel
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= a.n_atoms) return;  // warp-uniform
    const WinDev &W = a.win[a.atom_win[i]];
    const float L = W.box, h = W.hbox;
    const float4 xi = a.pos[i];
    const int trow = a.atype[i].x * a.n_lj_types;
    const int terms = ALL ? 7 : a.terms;
    const float epf = 1.0f - 1.0f / kEp;
    const float kfar = -2.0f * epf / 3.0f;
    const int n = min(a.row_n[i], a.row_cap);
    const int *row = a.rows + (long long)i * a.row_cap;
    long long fx = 0, fy = 0, fz = 0;
    for (int k = lane; k < n; k += 32) {
        const int e = row[k];
        const int j = e & INT_MAX;
        const float4 xj = a.pos[j];
        const float rx = mimg(xi.x - xj.x, L, h);
        const float ry = mimg(xi.y - xj.y, L, h);
        const float rz = mimg(xi.z - xj.z, L, h);
        const float d2 = dist2f(rx, ry, rz);
        if (!(d2 < a.cut2)) continue;
        const int2 ty = a.atype[j];
        const float ri = rsqrtf(d2);
        const float ri2 = ri * ri;
        const float qq = xi.w * xj.w;
        float fs = 0.0f;
        if (terms & 4) {
            const float rm = __ldg(a.rmax + ty.y);
            const float two = 2.0f * rm;
            const float r2 = rm * rm;
            fs = d2 > __fmul_rn(two, two) ? kfar * qq * ri2 * ri
                                          : -qq * (epf / (24.0f * r2 * r2)) * (8.0f * rm - 3.0f * d2 * ri);
        }
        if (e >= 0) {
            if (terms & 1) {
                const float2 ab = __ldg(a.ljab + trow + ty.x);
                const float r6 = ri2 * ri2 * ri2;
                fs += r6 * fmaf(12.0f * ab.x, r6, -6.0f * ab.y) * ri2;
            }
            if (terms & 2) fs += qq * ri2 * ri;
        }
        const float px = fs * rx, py = fs * ry, pz = fs * rz;
        check_force(a.status, px, py, pz);
        fx += to_fix(px);
        fy += to_fix(py);
        fz += to_fix(pz);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(kFull, fx, o);
        fy += __shfl_xor_sync(kFull, fy, o);
        fz += __shfl_xor_sync(kFull, fz, o);
    }
    if (lane == 0 && (fx | fy | fz)) {
        unsigned long long *acc = a.facc + 3 * (long long)i;
        atomicAdd(acc + 0, (unsigned long long)fx);
        atomicAdd(acc + 1, (unsigned long long)fy);
        atomicAdd(acc + 2, (unsigned long long)fz);
    }
}

unsigned atom_blocks(int n) { return (unsigned)((n + kNblThreads - 1) / kNblThreads); }
unsigned warp_blocks(int n) { return (unsigned)(((long long)n * 32 + kNblThreads - 1) / kNblThreads); }

}  // namespace

void launch_nblist_build(const NbListArgs &a, cudaStream_t s) {
    if (a.n_atoms <= 0) return;
    nbl_check_kernel<<<atom_blocks(a.n_atoms), kNblThreads, 0, s>>>(a);
    nbl_bin_kernel<<<atom_blocks(a.n_atoms), kNblThreads, 0, s>>>(a);
    nbl_scan_kernel<<<1, 1024, 0, s>>>(a);
    nbl_scatter_kernel<<<atom_blocks(a.n_atoms), kNblThreads, 0, s>>>(a);
    nbl_rows_kernel<<<warp_blocks(a.n_atoms), kNblThreads, 0, s>>>(a);
}

void launch_nblist_pairs(const NbListArgs &a, cudaStream_t s) {
    if (a.n_atoms <= 0) return;
    if (a.terms == 7) nbl_pairs_kernel<true><<<warp_blocks(a.n_atoms), kNblThreads, 0, s>>>(a);
    else nbl_pairs_kernel<false><<<warp_blocks(a.n_atoms), kNblThreads, 0, s>>>(a);
}

}  // namespace isspa
