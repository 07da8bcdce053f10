// tis_pair_lists_noalloc: the cell binning and SR/LR pair-list build of
// populate_lists (E:1461-1694 of src/16SCD_Mg_Cl_K_COPY_fast.cpp) for one
// configuration held in caller-owned device memory, without allocating.
//
// Why it exists: some callers cannot allocate device memory at the point they
// need a list.  A host whose CUDA work is being captured into a graph cannot
// call cudaMalloc (it is not a capturable operation), cudaFree synchronises the
// whole device, and engines that embed this library in their own time step often
// run under a fixed memory budget with every buffer reserved up front.  This
// entry point therefore takes only caller buffers and keeps its scratch (cell
// counts, offsets and the cell-sorted particle list) in a file-scope __device__
// array that every GPU loading the library holds until the process exits.
//
// Limits: at most kNaMaxParticles particles and kNaMaxCells cells.  All calls
// share the one scratch array, so calls that overlap on the GPU (different
// streams, or different host threads on one device) race and must be ordered
// by the caller.  The first call on a device looks up the array's device
// address (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture begins.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "tis_device.cuh"
#include "tis_host.h"

namespace {

constexpr int kNaMaxParticles = 65536;
constexpr int kNaMaxCells = 32768;
constexpr int kNaThreads = 128;
// scratch layout (ints): count[kNaMaxCells] | start[kNaMaxCells] | fill[kNaMaxCells] |
//                        cell_of[kNaMaxParticles] | sorted[kNaMaxParticles]
constexpr size_t kNaScratchInts = 3 * (size_t)kNaMaxCells + 2 * (size_t)kNaMaxParticles;  // 896 KiB

static __device__ __align__(256) int g_na_scratch[kNaScratchInts];

struct NaArgs {
    const double *x, *y, *z;
    const int *kind;
    int n;
    double box[3], hbox[3], lcell[3];
    int mc[3], nc;
    double r2sr, r2lr;
    int *sr, *lr;
    long long sr_cap, lr_cap;
    unsigned long long *counts;  // caller's device [SR pairs, LR pairs, particles outside the grid]
    int *scratch;
};

__device__ inline int na_axis(double v, double side, double l)
{
    double t = v;
    if (t < 0) t = __dadd_rn(t, side);
    else if (t > side) t = __dsub_rn(t, side);
    return (int)ceil(__ddiv_rn(t, l));
}

__global__ void k_na_assign(NaArgs a)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    int *count = a.scratch, *cell_of = a.scratch + 3 * kNaMaxCells;
    const int i1 = na_axis(a.x[p], a.box[0], a.lcell[0]);
    const int i2 = na_axis(a.y[p], a.box[1], a.lcell[1]);
    const int i3 = na_axis(a.z[p], a.box[2], a.lcell[2]);
    if (i1 < 1 || i1 > a.mc[0] || i2 < 1 || i2 > a.mc[1] || i3 < 1 || i3 > a.mc[2]) {
        cell_of[p] = -1;  // beyond the single periodic wrap of separate_in_cells: left out, and counted
        atomicAdd(a.counts + 2, 1ull);
        return;
    }
    const int c = (i1 - 1) * a.mc[1] * a.mc[2] + (i2 - 1) * a.mc[2] + (i3 - 1);
    cell_of[p] = c;
    atomicAdd(count + c, 1);
}

__global__ void k_na_scan(NaArgs a)  // one block: exclusive scan of the cell counts
{
    int *count = a.scratch, *start = a.scratch + kNaMaxCells;
    __shared__ int s_carry, s_warp[32];
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int base = 0; base < a.nc; base += blockDim.x) {
        const int c = base + threadIdx.x;
        const int v = c < a.nc ? count[c] : 0;
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_warp[w] = incl;
        __syncthreads();
        if (w == 0) {
            int t = lane < nw ? s_warp[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += u;
            }
            if (lane < nw) s_warp[lane] = t;
        }
        __syncthreads();
        const int excl = s_carry + (w > 0 ? s_warp[w - 1] : 0) + incl - v;
        if (c < a.nc) start[c] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry = excl + v;
        __syncthreads();
    }
}

__global__ void k_na_fill(NaArgs a)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    int *start = a.scratch + kNaMaxCells, *fill = a.scratch + 2 * kNaMaxCells;
    int *cell_of = a.scratch + 3 * kNaMaxCells, *sorted = cell_of + kNaMaxParticles;
    const int c = cell_of[p];
    if (c < 0) return;
    sorted[start[c] + atomicAdd(fill + c, 1)] = p;
}

__device__ inline double na_r2(const NaArgs &a, int i, int j)  // CC_vector + r^2 (E:674-683)
{
    double v[3] = {__dsub_rn(a.x[i], a.x[j]), __dsub_rn(a.y[i], a.y[j]), __dsub_rn(a.z[i], a.z[j])};
    for (int k = 0; k < 3; ++k) {
        if (v[k] > a.hbox[k]) v[k] = __dsub_rn(v[k], a.box[k]);
        if (v[k] < -a.hbox[k]) v[k] = __dadd_rn(v[k], a.box[k]);
    }
    return __dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2]));
}

// every unordered pair once (i < j): SR when r^2 <= r2sr, else LR when r^2 <= r2lr and
// neither bead is a sugar or a base (E:1626-1644)
__global__ void k_na_pairs(NaArgs a)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const int *count = a.scratch, *start = a.scratch + kNaMaxCells;
    const int *cell_of = a.scratch + 3 * kNaMaxCells, *sorted = cell_of + kNaMaxParticles;
    const int c = cell_of[p];
    if (c < 0) return;
    const int kp = a.kind[p];
    const bool chp = kp != 1 && kp != 2;
    const int ci[3] = {c / (a.mc[1] * a.mc[2]) + 1, (c / a.mc[2]) % a.mc[1] + 1, c % a.mc[2] + 1};
    int nb[3][3], nn[3];
    for (int ax = 0; ax < 3; ++ax) {
        nn[ax] = 0;
        for (int dd = -1; dd <= 1; ++dd) {
            int v = ci[ax] + dd;
            if (v < 1) v += a.mc[ax];
            if (v > a.mc[ax]) v -= a.mc[ax];
            bool dup = false;
            for (int t = 0; t < nn[ax]; ++t) dup |= nb[ax][t] == v;
            if (!dup) nb[ax][nn[ax]++] = v;
        }
    }
    for (int u = 0; u < nn[0]; ++u)
        for (int v = 0; v < nn[1]; ++v)
            for (int w = 0; w < nn[2]; ++w) {
                const int cc = (nb[0][u] - 1) * a.mc[1] * a.mc[2] + (nb[1][v] - 1) * a.mc[2] + (nb[2][w] - 1);
                for (int t = 0; t < count[cc]; ++t) {
                    const int j = sorted[start[cc] + t];
                    if (j <= p) continue;
                    const double r2 = na_r2(a, p, j);
                    const int kj = a.kind[j];
                    if (r2 <= a.r2sr) {
                        const unsigned long long s = atomicAdd(a.counts, 1ull);
                        if ((long long)s < a.sr_cap) { a.sr[2 * s] = p; a.sr[2 * s + 1] = j; }
                    } else if (r2 <= a.r2lr && chp && kj != 1 && kj != 2) {
                        const unsigned long long s = atomicAdd(a.counts + 1, 1ull);
                        if ((long long)s < a.lr_cap) { a.lr[2 * s] = p; a.lr[2 * s + 1] = j; }
                    }
                }
            }
}

std::mutex g_na_mutex;
int *g_na_ptr[64] = {nullptr};

}  // namespace

extern "C" int tis_pair_lists_noalloc(const double *d_x, const double *d_y, const double *d_z, const int32_t *d_kind,
                                      int32_t n, const double *box, double sr_radius, double lr_radius,
                                      int32_t *d_sr_pairs, int64_t sr_cap, int32_t *d_lr_pairs, int64_t lr_cap,
                                      uint64_t *d_counts, void *stream)
{
    using tis::fail;
    if (!d_x || !d_y || !d_z || !d_kind || !box || !d_counts || n < 0 || sr_cap < 0 || lr_cap < 0 ||
        (sr_cap > 0 && !d_sr_pairs) || (lr_cap > 0 && !d_lr_pairs))
        return fail(TIS_ERR_ARG, "tis_pair_lists_noalloc: bad argument");
    if (!(sr_radius > 0) || !(lr_radius >= sr_radius))
        return fail(TIS_ERR_ARG, "tis_pair_lists_noalloc: need 0 < sr_radius <= lr_radius");
    if (n > kNaMaxParticles)
        return fail(TIS_ERR_ARG, "tis_pair_lists_noalloc: %d particles exceed the fixed limit of %d", n, kNaMaxParticles);
    NaArgs a;
    memset(&a, 0, sizeof a);
    a.nc = 1;
    for (int k = 0; k < 3; ++k) {
        if (!(box[k] > 0)) return fail(TIS_ERR_ARG, "tis_pair_lists_noalloc: box side %d not positive", k);
        a.box[k] = box[k];
        a.hbox[k] = 0.5 * box[k];
        a.mc[k] = (int)(box[k] / lr_radius);  // E:1484-1490
        if (a.mc[k] < 1) return fail(TIS_ERR_ARG, "tis_pair_lists_noalloc: box side %d below the LR radius", k);
        a.lcell[k] = box[k] / a.mc[k];
        if ((long long)a.nc * a.mc[k] > kNaMaxCells)
            return fail(TIS_ERR_ARG, "tis_pair_lists_noalloc: more than %d cells; use a larger LR radius or smaller box",
                        kNaMaxCells);
        a.nc *= a.mc[k];
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(TIS_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(TIS_ERR_ARG, "tis_pair_lists_noalloc: device %d out of range", dev);
    {
        std::lock_guard<std::mutex> lk(g_na_mutex);
        if (!g_na_ptr[dev]) {  // set-up, once per device, with that device current
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_na_scratch);
            if (e != cudaSuccess) return fail(TIS_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            g_na_ptr[dev] = (int *)ptr;
        }
    }
    a.scratch = g_na_ptr[dev];
    a.x = d_x;
    a.y = d_y;
    a.z = d_z;
    a.kind = d_kind;
    a.n = n;
    a.r2sr = sr_radius * sr_radius;
    a.r2lr = lr_radius * lr_radius;
    a.sr = d_sr_pairs;
    a.lr = d_lr_pairs;
    a.sr_cap = sr_cap;
    a.lr_cap = lr_cap;
    a.counts = (unsigned long long *)d_counts;
    cudaStream_t s = (cudaStream_t)stream;
    // the shared scratch keeps the last call's contents: clear the counters that must start at zero
    if ((e = cudaMemsetAsync(a.scratch, 0, sizeof(int) * a.nc, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(a.scratch + 2 * kNaMaxCells, 0, sizeof(int) * a.nc, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_counts, 0, 3 * sizeof(uint64_t), s)) != cudaSuccess)
        return fail(TIS_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    if (n == 0) return TIS_OK;
    const int nb = (n + kNaThreads - 1) / kNaThreads;
    k_na_assign<<<nb, kNaThreads, 0, s>>>(a);
    k_na_scan<<<1, 256, 0, s>>>(a);
    k_na_fill<<<nb, kNaThreads, 0, s>>>(a);
    k_na_pairs<<<nb, kNaThreads, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TIS_ERR_CUDA, "tis_pair_lists_noalloc launch: %s", cudaGetErrorString(e));
    return TIS_OK;
}
