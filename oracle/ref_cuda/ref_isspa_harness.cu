// ref_isspa_harness.cu -- runs the reference's own IS-SPA field and force
// kernels (src/isspa_force_cuda.cu:110-327 of mccullaghlab/ISSPA-Force-Cuda,
// staged unmodified into oracle/_ref/src by oracle/ref_omp/build_ref.py) on MC
// points supplied by the caller, so that the engine and the reference CUDA
// path can be compared on the same point set.  Test infrastructure only.
//
// The reference's MC-point kernel and curand states are not used: the caller's
// points are written to mcpos with w = 1 (what isspa_MC_points_kernel leaves,
// isspa_force_cuda.cu:101-102), then the field and force kernels run with the
// launch shapes of isspa_grid_block (:362-408).  Every buffer is allocated to
// cover what those grids touch (the bounds argument):
//   * field kernel: threads with atom2 >= nAtoms only add zeros into
//     mcpos/enow/e0now[MC] with MC < nAtoms*nMC; table reads stay below
//     jt*nGRs + nGRs (density) and (nTypes-1)*nERs + nGRs (field table, which
//     the kernel indexes with the density bin), and the field table is
//     allocated to that length;
//   * force kernel: forceTable[jt*nRs + bin + 1] reaches nTypes*nRs when bin =
//     nRs-1 (one past the table), so the table gets one extra zero; the bin is
//     non-negative whenever forceR0 < 1.5 forceDR (checked below); lane 0 of
//     every warp of the rounded-up grid adds into f[atom] with atom up to
//     (forceGridSize*1024-1)/forceThreads, so f has that many rows.
// Usage: ref_isspa_harness <input> <output>.  Input (little-endian):
//   int32[8]  nAtoms, nMC, nTypes, nRs, nGRs, nERs, runs, 0
//   float[7]  box, forceR0, forceDR, gR0, gDR, eR0, eDR
//   float xyz[nAtoms][4], int32 types[nAtoms], float rmax[nTypes], vtot[nTypes],
//   float g[nTypes*nGRs], e[nTypes*nERs], f[nTypes*nRs], pts[nAtoms*nMC][3]
// Output: float forces[runs][nAtoms][4], each run from zeroed accumulators.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define __shfl_down(v, o) __shfl_down_sync(0xffffffffu, (v), (o))
#include "isspa_force_cuda.cu"

namespace {

bool ok(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    return false;
}

template <typename T>
bool read_n(FILE *f, std::vector<T> &v, size_t n) {
    v.resize(n);
    return n == 0 || std::fread(v.data(), sizeof(T), n, f) == n;
}

template <typename T>
T *dev(const std::vector<T> &h, size_t n_alloc) {
    T *p = nullptr;
    if (!ok(cudaMalloc(&p, sizeof(T) * std::max<size_t>(n_alloc, 1)), "cudaMalloc")) std::exit(3);
    if (!ok(cudaMemset(p, 0, sizeof(T) * std::max<size_t>(n_alloc, 1)), "cudaMemset")) std::exit(3);
    if (!h.empty() && !ok(cudaMemcpy(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice), "cudaMemcpy"))
        std::exit(3);
    return p;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s input output\n", argv[0]);
        return 2;
    }
    FILE *in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int hdr[8];
    float prm[7];
    if (std::fread(hdr, sizeof(int), 8, in) != 8 || std::fread(prm, sizeof(float), 7, in) != 7) return 2;
    const int N = hdr[0], M = hdr[1], nt = hdr[2], nR = hdr[3], nG = hdr[4], nE = hdr[5], runs = hdr[6];
    const long long P = (long long)N * M;
    // preconditions of the bounds argument and of the reference's int / float index arithmetic
    const long long field_threads = ((N + 31) / 32) * 32LL;
    if (N <= 0 || M <= 0 || nt <= 0 || nR < 2 || nG < 2 || nE < 2 || runs <= 0 || runs > 64 ||
        field_threads * P >= (1LL << 31) || P * N >= (1LL << 24) || !(prm[1] < 1.5f * prm[2]) || !(prm[0] > 0.f)) {
        std::fprintf(stderr, "input outside the harness's checked range\n");
        return 2;
    }
    std::vector<float4> xyz;
    std::vector<int> types;
    std::vector<float> rmax, vtot, g, e, f, pts;
    if (!read_n(in, xyz, N) || !read_n(in, types, N) || !read_n(in, rmax, nt) || !read_n(in, vtot, nt) ||
        !read_n(in, g, (size_t)nt * nG) || !read_n(in, e, (size_t)nt * nE) || !read_n(in, f, (size_t)nt * nR) ||
        !read_n(in, pts, (size_t)P * 3))
        return 2;
    std::fclose(in);
    for (int t : types)
        if (t < 0 || t >= nt) return 2;

    isspa s;
    std::memset(&s, 0, sizeof s);
    s.nTypes = nt;
    s.nMC = M;
    s.nRs = nR;
    s.nGRs = nG;
    s.nERs = nE;
    s.forceRparams = make_float2(prm[1], prm[2]);
    s.gRparams = make_float2(prm[3], prm[4]);
    s.eRparams = make_float2(prm[5], prm[6]);
    isspa_grid_block(N, N * N, prm[0], s);
    if (!ok(cudaGetLastError(), "isspa_grid_block")) return 3;
    // the force kernel forms MC = index - atom * nThreads in float: exact below 2^24
    if ((long long)s.forceGridSize * s.forceBlockSize > (1LL << 24)) {
        std::fprintf(stderr, "force grid beyond the reference's exact float index range\n");
        return 2;
    }

    const long long f_rows = std::max<long long>(N, ((long long)s.forceGridSize * s.forceBlockSize - 1) / s.forceThreads + 1);
    const size_t e_len = std::max<size_t>((size_t)nt * nE, (size_t)(nt - 1) * nE + nG);
    float4 *xyz_d = dev(xyz, N);
    int *types_d = dev(types, N);
    float *rmax_d = dev(rmax, nt), *vtot_d = dev(vtot, nt);
    float *g_d = dev(g, (size_t)nt * nG), *e_d = dev(e, e_len), *f_d = dev(f, (size_t)nt * nR + 1);
    std::vector<float4> mc(P);
    for (long long p = 0; p < P; ++p) mc[p] = make_float4(pts[3 * p], pts[3 * p + 1], pts[3 * p + 2], 1.0f);
    std::vector<float4> none;
    float4 *mcpos_d = dev(none, P), *enow_d = dev(none, P), *e0now_d = dev(none, P);
    float4 *frc_d = dev(none, f_rows), *isspaf_d = dev(none, N);
    std::vector<float> out((size_t)runs * N * 4);
    for (int r = 0; r < runs; ++r) {
        if (!ok(cudaMemcpy(mcpos_d, mc.data(), sizeof(float4) * P, cudaMemcpyHostToDevice), "points") ||
            !ok(cudaMemset(enow_d, 0, sizeof(float4) * P), "enow") ||
            !ok(cudaMemset(e0now_d, 0, sizeof(float4) * P), "e0now") ||
            !ok(cudaMemset(frc_d, 0, sizeof(float4) * f_rows), "forces"))
            return 3;
        isspa_field_kernel<<<s.fieldGridSize, s.fieldBlockSize>>>(xyz_d, rmax_d, types_d, g_d, e_d, enow_d, e0now_d,
                                                                  mcpos_d, s.fieldThreads);
        isspa_force_kernel<<<s.forceGridSize, s.forceBlockSize>>>(xyz_d, vtot_d, rmax_d, types_d, f_d, frc_d, enow_d,
                                                                  e0now_d, mcpos_d, (float)s.forceThreads, isspaf_d);
        if (!ok(cudaDeviceSynchronize(), "kernels") ||
            !ok(cudaMemcpy(out.data() + (size_t)r * N * 4, frc_d, sizeof(float4) * N, cudaMemcpyDeviceToHost),
                "read forces"))
            return 3;
    }
    FILE *o = std::fopen(argv[2], "wb");
    if (!o || std::fwrite(out.data(), sizeof(float), out.size(), o) != out.size()) return 2;
    std::fclose(o);
    return 0;
}
