// Device-side types and math shared by the TIS kernels (sm_103a).
//
// Precision policy (mixed mode): pair, bonded, stacking and hydrogen-bond
// geometry in FP32 from EXACT integer coordinate differences (positions are
// also kept as 32-bit fixed point over the periodic box, so a difference is an
// exact int32 whose wrap-around is the minimum image); every force
// contribution is converted to 64-bit fixed point (2^-32 kcal/mol/A) before it
// is summed, so sums are order-independent and deterministic; integration,
// thermostat and energy sums in FP64.  FP64 mode evaluates everything in FP64
// from the FP64 positions with the reference's own image convention.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace tis {

constexpr int kBlock = 128;          // particles per block; replicas are padded to it
constexpr int kNoise = 3000;         // shared Gaussians per step (E:2598)
constexpr int kNE = 11;              // energies vector (tis_energy_index)
constexpr double kSig0 = 1.5852;     // LJ length scale (E:749-821)
constexpr double kFixScale = 4294967296.0;   // 2^32 fixed-point units per kcal/mol/A
constexpr float kFixScaleF = 4294967296.0f;
constexpr float kFixLimit = 1.0e9f;  // |contribution| clamp (int64 range / 2^32 with margin)
constexpr int kExcl = 8;             // bonded (1-2, 1-3) partners stored per particle
constexpr int kExclShift = 30;       // SR list entry: partner | (exclusion multiplicity << 30)
constexpr int kIdxMask = (1 << kExclShift) - 1;
constexpr int kLanes = 4;            // neighbour-list slots per chunk (nb_idx)
constexpr int kLanesSR = 1;          // threads per particle in the SR pair kernel (lists of a few pairs)
constexpr int kLanesLR = 4;          // threads per particle in the LR pair kernel
constexpr int kThreadsLR = 512;      // threads per LR block (its kBlock particles in kBlock * 4 / 512 passes)
constexpr int kIntPer = 1;           // particles per thread in the integrator

// neighbour slot k of particle p: chunks of four slots per particle, chunk-major,
// so the four threads of a particle read 16 contiguous bytes and a warp 128
__host__ __device__ inline size_t nb_idx(int k, int p, int P)
{
    return (((size_t)(k >> 2) * (size_t)P + (size_t)p) << 2) + (size_t)(k & 3);
}

enum ErrBits : int { kErrCapacity = 1, kErrNonFinite = 2, kErrRange = 4 };

// Per-replica constants (uploaded once).
struct RepParams {
    double box[3], hbox[3], qinv[3], lcell[3];
    float qstep[3];
    int mc[3];
    int c0, nc;                  // first cell, number of cells
    int p0, n, npad, center;     // first particle, particles, padded, recentring bead (global)
    int nrna;                    // particles [p0, p0+nrna) are RNA beads
    int lr_interval;
    double T, h, lB, rc2, r2sr, r2lr, skin;
    float rc2f, r2srf, r2lrf, Tf;
    double kappa;                // inverse Debye length of the screened Coulomb term (0: unscreened, the reference)
    float kappaf;
    double mass[10], k1[10], k2[10], sigma[10], vcap[10];
    double k2fix[10], k2sig[10];  // K2 * 2^-32 (fixed-point force to velocity), K2 * sigma (noise)
    // pair tables, 1..45 (E:2908-2938); dm = D_LJ - 1.5852
    float dlj2[46], dm[46], flj[46], elj[46], d2min[46], qclb[46];
    float ljkeep2[46];           // (D_LJ + skin)^2 with a 1e-5 margin: pruned-list radius of uncharged pairs
    double dlj2_d[46], dlj_d[46], flj_d[46], elj_d[46], d2min_d[46], qclb_d[46];
    unsigned long long seed;
    int bt0, bt1, s30, s31, s20, s21, hb0, hb1, hba0, hba1, ca0, ca1;
    int kscr0, maxk;             // hb_K scratch offset and size
    int pk0;                     // first value of the replica in the group's packed (unpadded) host arrays
};

// Per-replica dynamic state.
struct RepState {
    long long klok, rebuilds;
    unsigned long long ctr;      // rand() draws consumed
    unsigned long long maxd2;    // bit pattern of max |x - x_old|^2 (non-negative double)
    double progress;
    int rebuild, lr_now, err, n_active;
    double e2hb, e3hb, e2st, e3st;
    double e2st_acc, e3st_acc;   // stacking energies being summed in the current step
    unsigned blocks_done;        // integrator blocks finished this step (the last one runs the skin check)
    unsigned pad_;
};

// ---- Philox-4x32-10 (Salmon et al., SC'11) --------------------------------
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[1] = (uint32_t)p1;
        c[3] = (uint32_t)p0;
        c[0] = n0;
        c[2] = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Draw k of the rand() stream of a replica: an integer in [1, 2^31-1].
__host__ __device__ inline uint32_t rand_value(unsigned long long seed, unsigned long long k)
{
    unsigned long long blk = k >> 2;
    uint32_t c[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), 0u, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    uint32_t v = c[k & 3u] >> 1;
    return v ? v : 1u;
}

// v / (2^31 - 1) rounded to nearest double, for 1 <= v <= 2^31 - 1: the reference's
// uniform (double) rand () / RAND_MAX from integer operations.  The binary expansion
// of v / (2^31 - 1) is the 31-bit pattern of v repeated without end, so the 53
// leading bits and the rounding bit come from at most three copies of it, and the
// bits beyond are never all zero: rounding to nearest adds the rounding bit.
__host__ __device__ inline double u31_ratio(uint32_t v)
{
    if (v >= 2147483647u) return 1.0;
#ifdef __CUDA_ARCH__
    const int s = 32 - __clz((int)v);  // significant bits of v
#else
    const int s = 32 - __builtin_clz(v);
#endif
    unsigned long long m = ((unsigned long long)v << 31) | v;  // the expansion from its leading one: s + 31 bits
    int len = s + 31;
    if (len < 54) {  // append the next copy's leading bits
        m = (m << (54 - len)) | ((unsigned long long)v >> (31 - (54 - len)));
        len = 54;
    }
    const unsigned long long b54 = m >> (len - 54);
    const unsigned long long mant = (b54 >> 1) + (b54 & 1ull);  // below 2^53: only v = 2^31 - 1 rounds up to it
    const unsigned long long bits = ((unsigned long long)(1023 - (31 - s) - 1) << 52) | (mant & ((1ull << 52) - 1ull));
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)bits);
#else
    double out;
    memcpy(&out, &bits, sizeof out);
    return out;
#endif
}

// ceil(u n) clamped to [1, n] as the reference picks a list entry, for u = v / (2^31 - 1)
// and 1 <= n < 2^20: v n / (2^31 - 1) is never an integer for v < 2^31 - 1 (the divisor
// is prime) and lies at least 2^-31 from one, far beyond the FP64 rounding of u and u n.
// The quotient floor(x / (2^31 - 1)) for x < 2^62 is (x + (x >> 31) + 1) >> 31: with
// x = q (2^31 - 1) + r, x >> 31 is q when r >= q and q - 1 when r < q, and either way
// the sum is q 2^31 plus a remainder below 2^31.
__host__ __device__ inline int pick_index(uint32_t v, int n)
{
    if (v >= 2147483647u) return n;
    const unsigned long long x = (unsigned long long)v * (unsigned)n;
    return (int)((x + (x >> 31) + 1ull) >> 31) + 1;
}

#ifdef __CUDACC__
// u < exp((ea - eb) / T) for u = v / (2^31 - 1), the Metropolis test of the H-bond
// Monte Carlo (E:2290-2300).  Decided in FP32 when u lies outside a margin around the
// FP32 estimate that covers its rounding (relative 1e-6 + 4e-7 |x|); else in FP64 as
// written.  Identical to the FP64 test for every input.
__device__ inline bool accept_move(uint32_t v, double ea, double eb, double T, float inv_t)
{
    const float x = (float)(ea - eb) * inv_t;
    const float ef = expf(x);
    const float uf = (float)v * (1.0f / 2147483647.0f);
    const float m = 1.0e-6f + 4.0e-7f * fabsf(x);
    if (uf < ef * (1.0f - m)) return true;
    if (uf > ef * (1.0f + m)) return false;
    return u31_ratio(v) < exp((ea - eb) / T);
}

// sqrt(-2 ln u) for u = v / (2^31-1), accurate in FP32 over the whole range.
__device__ inline float bm_radius(uint32_t v)
{
    const float inv = 1.0f / 2147483647.0f;
    float lg;
    if (v < 1073741824u) lg = logf((float)v * inv);
    else lg = log1pf(-(float)(2147483647u - v) * inv);
    return sqrtf(-2.0f * lg);
}

// ---- fixed point ----------------------------------------------------------
// round(v * 2^32) as int64 from 32-bit conversions only (64-bit conversions run
// on GB300's narrow FP64 pipe).  For |v| < 0.5 the product fits int32 and is
// rounded to nearest; for |v| >= 0.5, v is a multiple of 2^-24, so the split
// v = floor(v) + frac is exact and frac * 2^32 is an exact integer below 2^32.
// The result equals __float2ll_rn(v * 2^32) for every |v| < kFixLimit.
__device__ inline long long to_fix(float v, int &err)
{
    if (!(fabsf(v) < kFixLimit)) {
        if (v != v) { err |= kErrNonFinite; return 0; }
        err |= kErrNonFinite;
        v = v > 0 ? kFixLimit : -kFixLimit;
    }
    if (fabsf(v) < 0.5f) return (long long)__float2int_rn(v * kFixScaleF);
    const float hi = floorf(v);
    const unsigned lo = __float2uint_rz((v - hi) * kFixScaleF);
    return (long long)((unsigned long long)(long long)__float2int_rz(hi) << 32) + (long long)lo;
}

__device__ inline void atomic_add_fix(unsigned long long *a, long long v)
{
    atomicAdd(a, (unsigned long long)v);
}

__device__ inline int jn12(int a, int b)  // E:1803-1805
{
    if (a < b) return (a - 1) * 9 - (a - 1) * a / 2 + b;
    return (b - 1) * 9 - (b - 1) * b / 2 + a;
}

#endif  // __CUDACC__

template <class R>
struct V3 {
    R x, y, z;
};
#ifdef __CUDACC__
template <class R>
__device__ inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R>
__device__ inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R>
__device__ inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R>
__device__ inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R>
__device__ inline V3<R> cross(V3<R> a, V3<R> b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

#endif  // __CUDACC__

}  // namespace tis
