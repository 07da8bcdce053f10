// Adjoint kernels of the TIS step (no counterpart in the reference, which has no
// derivatives): dU/dtheta of the potential at a state, and the reverse pass of one
// step of the fused Langevin update.
//
// The forces' Jacobian enters the reverse pass as J^T lambda.  Every force term is
// the exact negative gradient of its energy (LJ_FORCE of WCA_ENERGY, E:749-821;
// COULOMB_TRUNCATED_FORCE of its energy, E:825-855; the bonded, stacking and
// H-bond forces of their restraint energies, E:924-1454), so J is symmetric and
// J^T lambda = J lambda, the directional derivative of the force along lambda.
// It is evaluated by forward-mode differentiation: the force code of each term is
// written once more here over dual numbers (value, derivative along lambda), in
// FP64, with the discrete choices (cutoffs, Monte Carlo outcome, stack switching,
// dihedral imaging branch) taken from the values as the forward pass takes them.
//
// Parameter derivatives use that every parameter but the ion radii and the Debye
// length enters its terms as a factor (E_LJ = sqrt(ELJ_i ELJ_j); Q_C lB; st_E;
// hb_E), so lambda . dF/dtheta is lambda . F_term / theta times the factor's
// derivative; a radius moves the LJ contact distance D = R_i + R_j (dF/dD in
// closed form) and the ion's friction (K1, K2, sigma of E:2897-2903); the Debye
// length lambda_D of the screened Coulomb term U = C exp(-r / lambda_D) / r enters
// in closed form (dU/dlambda_D = C kappa^2 exp(-kappa r), d(F/r)/dlambda_D =
// C kappa^3 exp(-kappa r) / r with kappa = 1 / lambda_D; both vanish unscreened).
#include <cstdio>

#include "tis_kernels.cuh"

namespace tis {
namespace {

constexpr unsigned kFullMask = 0xffffffffu;
constexpr int kNP = kNParams;

// ---------------------------------------------------------------------------
// dual numbers: value and derivative along the tangent direction
// ---------------------------------------------------------------------------
template <class T>
struct DualT {
    T v, d;
};
template <class T>
__device__ inline DualT<T> operator+(DualT<T> a, DualT<T> b) { return {a.v + b.v, a.d + b.d}; }
template <class T>
__device__ inline DualT<T> operator-(DualT<T> a, DualT<T> b) { return {a.v - b.v, a.d - b.d}; }
template <class T>
__device__ inline DualT<T> operator-(DualT<T> a) { return {-a.v, -a.d}; }
template <class T>
__device__ inline DualT<T> operator*(DualT<T> a, DualT<T> b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
template <class T>
__device__ inline DualT<T> operator/(DualT<T> a, DualT<T> b)
{
    const T q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
template <class T>
__device__ inline DualT<T> operator+(DualT<T> a, T b) { return {a.v + b, a.d}; }
template <class T>
__device__ inline DualT<T> operator+(T a, DualT<T> b) { return {a + b.v, b.d}; }
template <class T>
__device__ inline DualT<T> operator-(DualT<T> a, T b) { return {a.v - b, a.d}; }
template <class T>
__device__ inline DualT<T> operator-(T a, DualT<T> b) { return {a - b.v, -b.d}; }
template <class T>
__device__ inline DualT<T> operator*(T a, DualT<T> b) { return {a * b.v, a * b.d}; }
template <class T>
__device__ inline DualT<T> operator/(T a, DualT<T> b)
{
    const T q = a / b.v;
    return {q, -q * b.d / b.v};
}
template <class T>
__device__ inline DualT<T> dsqrt(DualT<T> a)
{
    const T s = sqrt(a.v);
    return {s, s > T(0) ? T(0.5) * a.d / s : T(0)};
}

// The restraint terms and the pair Jacobian of a mixed-precision engine run in
// FP32 duals (differences taken in FP64 first, sums in FP64); FP64 engines and
// the parameter derivatives in FP64 duals
using Dual = DualT<double>;
template <class T>
__device__ inline DualT<T> dexp(DualT<T> a)
{
    const T e = exp(a.v);
    return {e, e * a.d};
}
template <class T>
__device__ inline DualT<T> datan2(DualT<T> y, DualT<T> x)
{
    const T n = x.v * x.v + y.v * y.v;
    return {atan2(y.v, x.v), n > T(0) ? (x.v * y.d - y.v * x.d) / n : T(0)};
}

template <class T>
using DVT = V3<DualT<T>>;

// positions (FP64 arrays) with the tangent (3P, component-major) as derivative;
// differences are formed in FP64 and then rounded to T
template <class T>
struct APos {
    const double *x, *y, *z, *t;
    int P;
    // position(b) - position(a), raw difference (the bonded terms' convention)
    __device__ DVT<T> vec(int a, int b) const
    {
        const T dx = (T)(x[b] - x[a]), dy = (T)(y[b] - y[a]), dz = (T)(z[b] - z[a]);
        if (!t) return {{dx, T(0)}, {dy, T(0)}, {dz, T(0)}};
        return {{dx, (T)(t[b] - t[a])}, {dy, (T)(t[P + b] - t[P + a])}, {dz, (T)(t[2 * P + b] - t[2 * P + a])}};
    }
};

// Force contributions of one term evaluated at unit strength: the derivative
// part is summed per atom of the term (its atoms set first, at most kSlots) and,
// times the term's strength, added to jv once per atom by flush(); lambda . value
// is summed in w (lambda = the tangent direction).
constexpr int kSlots = 7;
template <class T>
struct AAcc {
    double *jv;
    const double *lam;
    int P;
    double scale;
    double w;
    int ids[kSlots];
    double acc[kSlots][3];
    __device__ void atoms(const int *a, int n)
    {
#pragma unroll
        for (int s = 0; s < kSlots; ++s) {
            ids[s] = s < n ? a[s] : -1;
            acc[s][0] = acc[s][1] = acc[s][2] = 0.0;
        }
    }
    __device__ void add(int i, DVT<T> g)
    {
        if (jv)
#pragma unroll
            for (int s = 0; s < kSlots; ++s)
                if (ids[s] == i) {  // a slot per atom: registers, no atomics until flush
                    acc[s][0] += (double)g.x.d;
                    acc[s][1] += (double)g.y.d;
                    acc[s][2] += (double)g.z.d;
                }
        if (lam) w += lam[i] * (double)g.x.v + lam[P + i] * (double)g.y.v + lam[2 * P + i] * (double)g.z.v;
    }
    __device__ void flush()
    {
        if (!jv) return;
#pragma unroll
        for (int s = 0; s < kSlots; ++s)
            if (ids[s] >= 0 && (acc[s][0] != 0.0 || acc[s][1] != 0.0 || acc[s][2] != 0.0)) {
                atomicAdd(jv + ids[s], scale * acc[s][0]);
                atomicAdd(jv + P + ids[s], scale * acc[s][1]);
                atomicAdd(jv + 2 * P + ids[s], scale * acc[s][2]);
            }
    }
};

template <class T>
__device__ inline DVT<T> neg(DVT<T> a) { return {-a.x, -a.y, -a.z}; }

// ---------------------------------------------------------------------------
// the restraint terms (E:924-1454) over dual numbers
// ---------------------------------------------------------------------------
template <class T>
__device__ DualT<T> angle_of(const APos<T> &P, int i1, int i2, int i3)
{
    const DVT<T> a = P.vec(i2, i1), b = P.vec(i2, i3);
    const DVT<T> w = cross(a, b);
    return datan2(dsqrt(dot(w, w)), dot(a, b));
}

template <class T>
__device__ DualT<T> dihedral_of(const APos<T> &P, int i1, int i2, int i3, int i4)
{
    const DVT<T> v1 = P.vec(i1, i2), v2 = P.vec(i2, i3), v3 = P.vec(i3, i4);
    const DVT<T> m = cross(v1, v2), n = cross(v2, v3);
    return datan2(dot(v1, n) * dsqrt(dot(v2, v2)), dot(m, n));
}

// force of V = k0 (r0 - r)^2 on i1, i2
template <class T>
__device__ void bond_force(const APos<T> &P, AAcc<T> &A, int i1, int i2, DualT<T> k0, double r0)
{
    const DVT<T> v = P.vec(i1, i2);
    const DualT<T> r = dsqrt(dot(v, v));
    const DualT<T> t = T(2) * k0 * ((T)r0 - r) / r;
    const DVT<T> g = t * v;
    A.add(i1, neg(g));
    A.add(i2, g);
}

// force of V = k0 (th0 - theta)^2 at i2; clamp: none once cos theta < -0.99995 (E:1138-1251)
template <class T>
__device__ void angle_force(const APos<T> &P, AAcc<T> &A, int i1, int i2, int i3, DualT<T> k0, double th0, bool clamp)
{
    const DVT<T> a = P.vec(i2, i1), b = P.vec(i2, i3);
    const DualT<T> aa = dot(a, a), bb = dot(b, b), ab = dot(a, b);
    if (clamp && ab.v / sqrt(aa.v * bb.v) < T(-0.99995)) return;
    const DVT<T> w = cross(a, b);
    const DualT<T> ww = dsqrt(dot(w, w));
    if (ww.v == T(0)) return;
    const DualT<T> th = datan2(ww, ab);
    const DualT<T> s = T(2) * k0 * ((T)th0 - th) / ww;
    const DVT<T> g1 = (s / aa) * cross(a, w);
    const DVT<T> g3 = (-s / bb) * cross(b, w);
    A.add(i1, g1);
    A.add(i2, neg(g1 + g3));
    A.add(i3, g3);
}

// force of V = k0 (psi0 - psi)^2 of the dihedral i1-i2-i3-i4 (E:1306-1454)
template <class T>
__device__ void dihedral_force(const APos<T> &P, AAcc<T> &A, int i1, int i2, int i3, int i4, DualT<T> k0,
                               double psi0)
{
    const DVT<T> v1 = P.vec(i1, i2), v2 = P.vec(i2, i3), v3 = P.vec(i3, i4);
    const DVT<T> m = cross(v1, v2), n = cross(v2, v3);
    const DualT<T> mm = dot(m, m), nn = dot(n, n), v22 = dot(v2, v2);
    if (mm.v == T(0) || nn.v == T(0)) return;
    const DualT<T> l2 = dsqrt(v22);
    const DualT<T> psi = datan2(dot(v1, n) * l2, dot(m, n));
    const DualT<T> c = T(2) * k0 * ((T)psi0 - psi);
    const DVT<T> g1 = (-c * l2 / mm) * m;
    const DVT<T> g4 = (c * l2 / nn) * n;
    const DualT<T> p = dot(v1, v2) / v22, q = dot(v3, v2) / v22;
    const DVT<T> g2 = (T(-1) - p) * g1 + q * g4;
    A.add(i1, g1);
    A.add(i2, g2);
    A.add(i3, neg(g1 + g2 + g4));
    A.add(i4, g4);
}

// native dihedral imaged to within pi of the current one (E:1999-2019)
__device__ inline int branch_of(double psi, double nat)
{
    const double pi = 3.14159265358979323846;
    if (fabs(psi - nat) <= pi) return 0;
    return (psi - nat > pi) ? 1 : -1;
}
__device__ inline double shifted(double nat, int br) { return nat + 2.0 * 3.14159265358979323846 * br; }

// the six-term native-geometry restraint sum q (E:1983-2056, E:2177-2231)
template <class T>
__device__ DualT<T> six_q(const APos<T> &P, const int *k, const double *nat, DualT<T> rdev, double init, int br[3])
{
    const DualT<T> t1 = angle_of(P, k[0], k[1], k[4]);
    const DualT<T> t2 = angle_of(P, k[3], k[4], k[1]);
    const DualT<T> p0 = dihedral_of(P, k[0], k[1], k[4], k[3]);
    const DualT<T> p1 = dihedral_of(P, k[4], k[1], k[0], k[2]);
    const DualT<T> p2 = dihedral_of(P, k[1], k[4], k[3], k[5]);
    br[0] = branch_of((double)p0.v, nat[3]);
    br[1] = branch_of((double)p1.v, nat[4]);
    br[2] = branch_of((double)p2.v, nat[5]);
    const DualT<T> d0 = p0 - (T)shifted(nat[3], br[0]), d1 = p1 - (T)shifted(nat[4], br[1]),
                   d2 = p2 - (T)shifted(nat[5], br[2]);
    DualT<T> q = (T)init + T(5) * rdev * rdev;
    q = q + T(1.5) * (t1 - (T)nat[1]) * (t1 - (T)nat[1]);
    q = q + T(1.5) * (t2 - (T)nat[2]) * (t2 - (T)nat[2]);
    q = q + T(0.15) * d0 * d0 + T(0.15) * d1 * d1 + T(0.15) * d2 * d2;
    return q;
}

// force of V = w q for the six-term restraint
template <class T>
__device__ void six_force(const APos<T> &P, AAcc<T> &A, const int *k, const double *nat, const int br[3], DualT<T> w)
{
    bond_force(P, A, k[1], k[4], T(5) * w, nat[0]);
    angle_force(P, A, k[0], k[1], k[4], T(1.5) * w, nat[1], true);
    angle_force(P, A, k[3], k[4], k[1], T(1.5) * w, nat[2], true);
    dihedral_force(P, A, k[0], k[1], k[4], k[3], T(0.15) * w, shifted(nat[3], br[0]));
    dihedral_force(P, A, k[4], k[1], k[0], k[2], T(0.15) * w, shifted(nat[4], br[1]));
    dihedral_force(P, A, k[1], k[4], k[3], k[5], T(0.15) * w, shifted(nat[5], br[2]));
}

template <class T>
__device__ inline DualT<T> distance(const APos<T> &P, int a, int b)
{
    const DVT<T> v = P.vec(a, b);
    return dsqrt(dot(v, v));
}

// ---------------------------------------------------------------------------
// parameter bookkeeping
// ---------------------------------------------------------------------------
// LJ epsilon class of a particle type (MAXIKEY order: 1 P, 2 S, 3-6 bases, 7 Mg, 8 Cl, 9 K)
__device__ inline int eps_param(int t)
{
    if (t == 1) return 6;
    if (t == 2) return 7;
    if (t <= 6) return 8;
    if (t == 7) return 9;
    if (t == 8) return 10;
    return 11;
}
__device__ inline int radius_param(int t) { return t == 7 ? 12 : t == 9 ? 13 : -1; }

// g[i] += v for a run-time i, the array kept in registers (a select per slot
// instead of an indexed store, which would place g in local memory)
template <int N>
__device__ inline void gadd(double (&g)[N], int i, double v)
{
#pragma unroll
    for (int c = 0; c < N; ++c) g[c] += (c == i) ? v : 0.0;
}

// sum of NV doubles over a block of blockDim.x threads (multiple of 32) into thread 0
template <int NV>
__device__ void block_reduce(double (&v)[NV], double *smem /* NV * 32 */)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(kFullMask, v[k], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) smem[k * 32 + warp] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            v[k] = lane < nw ? smem[k * 32 + lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(kFullMask, v[k], o);
        }
    }
}

// ---------------------------------------------------------------------------
// pair terms over the neighbour lists (SR_interactions_lists, LR_interactions_lists)
// ---------------------------------------------------------------------------
// One thread per particle over its full list (every pair appears in both
// partners' lists).  mode 0: dU/dtheta (each pair half from each side); mode 1:
// jv[p] += (J tan)_p and the parameter terms of lambda = tan.  The LR kernel in
// mode 1 runs only for replicas whose LR force was refreshed in the step.
template <bool LR, class T>
__global__ void __launch_bounds__(kBlock) k_adj_pair(Dev d, AdjDev a, const double *tan, int mode)
{
    using DT = DualT<T>;
    __shared__ double s_red[10 * 32];
    const int p = blockIdx.x * kBlock + threadIdx.x;
    const int r = d.blk_rep[blockIdx.x];
    const RepParams *R = d.rp + r;
    if (LR && mode == 1 && !a.rlr[r]) return;  // block-uniform
    const int P = d.P;
    const int4 qp = d.q[p];
    const int tp = qp.w & 0xff, kp = (qp.w >> 8) & 0xff, act = (qp.w >> 16) & 1;
    const bool chp = kp != 1 && kp != 2;
    double g[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // parameters 6 .. 15
    double jx = 0, jy = 0, jz = 0;
    if (act) {
        const int cnt = LR ? d.n_lr[p] : d.n_sr[p];
        const int *nbr = LR ? d.nbr_lr : d.nbr_sr;
        const double lx = tan ? tan[p] : 0.0, ly = tan ? tan[P + p] : 0.0, lz = tan ? tan[2 * P + p] : 0.0;
        const double eps_p = R->elj_d[jn12(tp, tp)];
        for (int k = 0; k < cnt; ++k) {
            const int raw = nbr[nb_idx(k, p, P)];
            const int j = raw & kIdxMask;
            const double ljw = LR ? 0.0 : (double)(1 - (raw >> kExclShift));
            const int4 qj = d.q[j];
            const int tj = qj.w & 0xff, kj = (qj.w >> 8) & 0xff;
            const int J = jn12(tp, tj);
            double v[3] = {a.px[p] - a.px[j], a.py[p] - a.py[j], a.pz[p] - a.pz[j]};
            for (int c = 0; c < 3; ++c) {
                if (v[c] > R->hbox[c]) v[c] -= R->box[c];
                if (v[c] < -R->hbox[c]) v[c] += R->box[c];
            }
            // cutoff decisions in FP64, as the forward pass decides them
            const double r2e = __dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2]));
            const bool lj = !LR && ljw != 0.0 && r2e <= R->dlj2_d[J];
            const bool cou = (LR || (chp && kj != 1 && kj != 2)) && r2e <= R->rc2;
            if (!lj && !cou) continue;
            const V3<DT> dv = {{(T)v[0], tan ? (T)(lx - tan[j]) : T(0)}, {(T)v[1], tan ? (T)(ly - tan[P + j]) : T(0)},
                               {(T)v[2], tan ? (T)(lz - tan[2 * P + j]) : T(0)}};
            const DT r2 = dot(dv, dv);
            const DT rr = dsqrt(r2);
            DT F = {T(0), T(0)};
            const double wl = lx * v[0] + ly * v[1] + lz * v[2];  // lambda_p . (x_p - x_j)
            if (lj) {
                const DT dr = rr + (T)(kSig0 - R->dlj_d[J]);
                const DT s = (T)kSig0 / dr;
                const DT s2 = s * s, s4 = s2 * s2, s8 = s4 * s4, s14 = s8 * s4 * s2;
                const double c0 = ljw * R->flj_d[J];
                const DT phi = (T)c0 * (s14 - s8) * dr / rr;
                F = F + phi;
                const double eps_j = R->elj_d[jn12(tj, tj)];
                const bool radius = !(tp <= 6 && tj <= 6);
                if (mode == 0) {
                    const double s6 = (double)s4.v * (double)s2.v, s12 = s6 * s6;
                    const double u = ljw * R->elj_d[J] * (s12 - 2.0 * s6 + 1.0);
                    if (eps_p > 0.0) gadd(g, eps_param(tp) - 6, 0.25 * u / eps_p);
                    if (eps_j > 0.0) gadd(g, eps_param(tj) - 6, 0.25 * u / eps_j);
                    if (radius) {
                        const double dud = 0.5 * ljw * 12.0 * R->elj_d[J] * (s12 - s6) / (double)dr.v;
                        const int ip = radius_param(tp), ij = radius_param(tj);
                        if (ip >= 0) gadd(g, ip - 6, dud);
                        if (ij >= 0) gadd(g, ij - 6, dud);
                    }
                } else {
                    if (eps_p > 0.0) gadd(g, eps_param(tp) - 6, wl * (double)phi.v / (2.0 * eps_p));
                    if (eps_j > 0.0) gadd(g, eps_param(tj) - 6, wl * (double)phi.v / (2.0 * eps_j));
                    if (radius) {
                        const double dphi = c0 * (13.0 * (double)s14.v - 7.0 * (double)s8.v) / (double)rr.v;
                        const int ip = radius_param(tp), ij = radius_param(tj);
                        if (ip >= 0) gadd(g, ip - 6, wl * dphi);
                        if (ij >= 0) gadd(g, ij - 6, wl * dphi);
                    }
                }
            }
            if (cou) {
                const double kap = R->kappa;
                DT psi;
                double u;  // the pair's Coulomb energy
                if (kap == 0.0) {
                    psi = (T)R->qclb_d[J] / (rr * r2);
                    u = R->qclb_d[J] / (double)rr.v;
                } else {  // screened: F / r = C exp(-kappa r) (1 + kappa r) / r^3
                    const DT ex = dexp((T)(-kap) * rr);
                    psi = (T)R->qclb_d[J] * ex * ((T)1 + (T)kap * rr) / (rr * r2);
                    u = R->qclb_d[J] * (double)ex.v / (double)rr.v;
                    const double ek = R->qclb_d[J] * (double)ex.v * kap * kap;  // dU/dlambda_D
                    if (mode == 0) g[9] += 0.5 * ek;
                    else g[9] += wl * ek * kap / (double)rr.v;
                }
                F = F + psi;
                if (R->lB != 0.0) {
                    if (mode == 0) g[8] += 0.5 * u / R->lB;
                    else g[8] += wl * (double)psi.v / R->lB;
                }
            }
            if (mode == 1) {  // d/dtan of F (x_p - x_j), summed in FP64
                jx += (double)F.d * v[0] + (double)F.v * (double)dv.x.d;
                jy += (double)F.d * v[1] + (double)F.v * (double)dv.y.d;
                jz += (double)F.d * v[2] + (double)F.v * (double)dv.z.d;
            }
        }
        if (mode == 1) {
            a.jv[p] += jx;
            a.jv[P + p] += jy;
            a.jv[2 * P + p] += jz;
        }
    }
    block_reduce<10>(g, s_red);
    if (threadIdx.x == 0)
        for (int k = 0; k < 10; ++k)
            if (g[k] != 0.0) atomicAdd(a.dth + r * kNP + 6 + k, g[k]);
}

// ---------------------------------------------------------------------------
// bonded terms, stacks and formed H-bonds, one thread per term
// ---------------------------------------------------------------------------
constexpr int kAdjTopoThreads = 128;

template <class T>
__global__ void __launch_bounds__(kAdjTopoThreads) k_adj_topo(Dev d, AdjDev a, const double *tan, int mode)
{
    using DT = DualT<T>;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int kind, item;
    if (t < d.nbt) { kind = 0; item = t; }
    else if (t < d.nbt + d.nst3) { kind = 1; item = t - d.nbt; }
    else if (t < d.nbt + d.nst3 + d.nst2) { kind = 2; item = t - d.nbt - d.nst3; }
    else if (t < d.nbt + d.nst3 + d.nst2 + a.nhb) { kind = 3; item = t - d.nbt - d.nst3 - d.nst2; }
    else return;
    if (kind == 0 && mode == 0) return;  // no parameter of this set enters the bonded terms
    if (kind == 3 && !a.rhb[item]) return;
    const APos<T> P{a.px, a.py, a.pz, mode == 1 ? tan : nullptr, d.P};
    AAcc<T> A{mode == 1 ? a.jv : nullptr, mode == 1 ? tan : nullptr, d.P, 1.0, 0.0, {}, {}};
    int r = 0, param = -1;
    double dE = 0.0, u1 = 0.0;
    if (kind == 0) {
        const int4 id = d.bt_idx[item];
        const double2 par = d.bt_par[item];
        const int at[3] = {id.x, id.y, id.z};
        A.atoms(at, id.w == 0 ? 2 : 3);
        const DT k0 = {(T)par.x, T(0)};
        if (id.w == 0) bond_force(P, A, id.x, id.y, k0, par.y);
        else angle_force(P, A, id.x, id.y, id.z, k0, par.y, false);
        A.flush();
        return;
    } else if (kind == 1) {  // tertiary: U = st_E / (1 + q), st_E = -st_D
        const int *id = d.st3_idx + 6 * item;
        const double *nat = d.st3_nat + 6 * item;
        r = d.rep_of[id[0]];
        int br[3];
        const DT rdev = distance(P, id[1], id[4]) - (T)nat[0];
        const DT Dn = six_q(P, id, nat, rdev, 1.0, br);
        u1 = 1.0 / (double)Dn.v;
        param = 4;
        dE = -1.0;
        if (mode == 1) {
            A.scale = d.st3_E[item];
            A.atoms(id, 6);
            six_force(P, A, id, nat, br, T(-1) / (Dn * Dn));
            A.flush();
        }
    } else if (kind == 2) {  // secondary: U = st_E / (1 + 1.4 dr^2 + 4 dpsi1^2 + 4 dpsi2^2)
        const int *id = d.st2_idx + 7 * item;
        r = d.rep_of[id[0]];
        for (int u = d.st2_offby_off[item]; u < d.st2_offby_off[item + 1]; ++u) {  // E:1960-1981
            const int k = d.st2_offby_idx[u];
            const int *tid = d.st3_idx + 6 * k;
            if ((double)distance(P, tid[1], tid[4]).v - d.st3_nat[6 * k] < 10.0) return;
        }
        const DT rr = distance(P, id[2], id[5]);
        const DT p1 = dihedral_of(P, id[0], id[1], id[3], id[4]);
        const DT p2 = dihedral_of(P, id[6], id[4], id[3], id[1]);
        const double p10 = shifted(-2.58684, branch_of((double)p1.v, -2.58684));
        const double p20 = shifted(3.07135, branch_of((double)p2.v, 3.07135));
        const double r0 = d.st2_r0[item];
        const DT Dn = T(1) + T(1.4) * (rr - (T)r0) * (rr - (T)r0) + T(4) * (p1 - (T)p10) * (p1 - (T)p10) +
                      T(4) * (p2 - (T)p20) * (p2 - (T)p20);
        u1 = 1.0 / (double)Dn.v;
        param = a.st2_cls[item];
        dE = a.st2_dss[item];
        if (mode == 1) {
            A.scale = d.st2_E[item];
            A.atoms(id, 7);
            const DT w = T(-1) / (Dn * Dn);
            bond_force(P, A, id[2], id[5], T(1.4) * w, r0);
            dihedral_force(P, A, id[0], id[1], id[3], id[4], T(4) * w, p10);
            dihedral_force(P, A, id[6], id[4], id[3], id[1], T(4) * w, p20);
            A.flush();
        }
    } else {  // formed H-bond: U = hb_E exp(-q)
        const int *id = d.hb_idx + 6 * item;
        const double *nat = d.hb_nat + 6 * item;
        r = d.rep_of[id[0]];
        int br[3];
        const DT rdev = distance(P, id[1], id[4]) - (T)nat[0];
        const DT q = six_q(P, id, nat, rdev, 0.0, br);
        const DT e = dexp(-q);
        u1 = (double)e.v;
        param = 5;
        dE = a.hb_dhs[item];
        if (mode == 1) {
            A.scale = d.hb_E[item];
            A.atoms(id, 6);
            six_force(P, A, id, nat, br, -e);
            A.flush();
        }
    }
    if (param < 0 || dE == 0.0) return;
    const double gval = mode == 0 ? u1 * dE : A.w * dE;
    if (gval != 0.0) atomicAdd(a.dth + r * kNP + param, gval);
}

// ---------------------------------------------------------------------------
// reverse pass of move_rigid_units (E:2660-2732, leap_frog_move_atom E:570-642,
// adjust_box E:2632-2656) with full_forces' noise (E:2612-2622)
// ---------------------------------------------------------------------------
// per replica: S = sum over particles of (lambda_x' + lambda_xo'), the adjoint of
// the recentring shift sh = box/2 - x'_centre that moves every x' and x_old'
__global__ void __launch_bounds__(kBlock) k_adj_center(Dev d, AdjDev a)
{
    __shared__ double s_red[3 * 32];
    const int p = blockIdx.x * kBlock + threadIdx.x;
    const int r = d.blk_rep[blockIdx.x];
    const int P = d.P;
    double v[3] = {0, 0, 0};
    if ((d.q[p].w >> 16) & 1)
        for (int c = 0; c < 3; ++c) v[c] = a.lam[c * P + p] + a.lam[(3 + c) * P + p];
    block_reduce<3>(v, s_red);
    if (threadIdx.x == 0)
        for (int c = 0; c < 3; ++c) atomicAdd(a.cen + 3 * r + c, v[c]);
}

// lambda of (x', x_old', v') after the step -> lambda of (x, x_old, v) before it,
// less the force path: lamf = K2 lambda_v' (the force's adjoint), mu += lamf
// (the LR force's adjoint since its refresh), jv = 0; the friction's dependence
// on the ion radii goes to dth
__global__ void __launch_bounds__(kBlock) k_adj_move(Dev d, AdjDev a)
{
    __shared__ double s_red[2 * 32];
    const int p = blockIdx.x * kBlock + threadIdx.x;
    const int r = d.blk_rep[blockIdx.x];
    const RepParams *R = d.rp + r;
    const int P = d.P;
    const int4 qp = d.q[p];
    double g[2] = {0, 0};
    if ((qp.w >> 16) & 1) {
        const int t = qp.w & 0xff;
        const double k1 = R->k1[t], k2 = R->k2[t], h = R->h;
        const double sg = d.noise == 0 ? R->sigma[t] : 0.0;
        const int kn = (p - R->p0 + 1) % 1000;
        double v0[3], f[3], gn[3], vp[3], A[3], lvpp[3], lvp[3];
        for (int c = 0; c < 3; ++c) {
            v0[c] = a.rx[(6 + c) * P + p];
            f[c] = a.rf[c * P + p];
            gn[c] = a.rg[r * kNoise + kn + 1000 * c];
            vp[c] = k1 * v0[c] + k2 * (f[c] + sg * gn[c]);
            A[c] = a.lam[c * P + p] - (p == R->center ? a.cen[3 * r + c] : 0.0);
            lvpp[c] = a.lam[(6 + c) * P + p] + h * A[c];
        }
        const double vv = vp[0] * vp[0] + vp[1] * vp[1] + vp[2] * vp[2];
        const double vsq = R->vcap[t] * vv;
        if (vsq > 1.0) {  // v'' = v' / sqrt(vcap |v'|^2): Jacobian (I - u u^T) / sqrt(vsq)
            const double inv = 1.0 / sqrt(vv), nrm = sqrt(vsq);
            const double u[3] = {vp[0] * inv, vp[1] * inv, vp[2] * inv};
            const double ul = u[0] * lvpp[0] + u[1] * lvpp[1] + u[2] * lvpp[2];
            for (int c = 0; c < 3; ++c) lvp[c] = (lvpp[c] - u[c] * ul) / nrm;
        } else {
            for (int c = 0; c < 3; ++c) lvp[c] = lvpp[c];
        }
        for (int c = 0; c < 3; ++c) {
            const double lxo = a.lam[(3 + c) * P + p];
            a.lam[c * P + p] = 2.0 * A[c] + lxo;
            a.lam[(3 + c) * P + p] = -A[c];
            a.lam[(6 + c) * P + p] = k1 * lvp[c] - h * A[c];
            const double lf = k2 * lvp[c];
            a.lamf[c * P + p] = lf;
            a.mu[c * P + p] += lf;
            a.jv[c * P + p] = 0.0;
        }
        const int rp = radius_param(t);
        if (rp >= 0) {  // VISC = 0.555 RLJ; K1 = exp(-VISC h / m); K2 = (1 - K1) / VISC; sigma = sqrt(2 VISC T / h)
            const double visc = (1.0 - k1) / k2, m = R->mass[t];
            const double dk1 = -k1 * h / m * 0.555;
            const double dk2 = 0.555 * (k1 * h * visc / m - (1.0 - k1)) / (visc * visc);
            const double dsg = sg > 0.0 ? 0.555 * sg / (2.0 * visc) : 0.0;
            double s = 0.0;
            for (int c = 0; c < 3; ++c) s += lvp[c] * (dk1 * v0[c] + dk2 * (f[c] + sg * gn[c]) + k2 * dsg * gn[c]);
            g[rp - 12] = s;
        }
    }
    block_reduce<2>(g, s_red);
    if (threadIdx.x == 0) {
        if (g[0] != 0.0) atomicAdd(a.dth + r * kNP + 12, g[0]);
        if (g[1] != 0.0) atomicAdd(a.dth + r * kNP + 13, g[1]);
    }
}

// lambda_x += J^T lamf (+ J_LR^T mu where the LR force was refreshed; mu then restarts)
__global__ void __launch_bounds__(kBlock) k_adj_finish(Dev d, AdjDev a)
{
    const int p = blockIdx.x * kBlock + threadIdx.x;
    const int r = d.blk_rep[blockIdx.x];
    const int P = d.P;
    for (int c = 0; c < 3; ++c) {
        a.lam[c * P + p] += a.jv[c * P + p];
        if (a.rlr[r]) a.mu[c * P + p] = 0.0;
    }
}

// the step's inputs, after its forces and before its integrator: x .. v, the force
// (f + the held LR force, without the noise) in FP64, the LR refresh flag
__global__ void __launch_bounds__(kBlock) k_adj_record(Dev d, AdjDev a)
{
    const int p = blockIdx.x * kBlock + threadIdx.x;
    const int P = d.P;
    const double *src[9] = {d.x, d.y, d.z, d.xo, d.yo, d.zo, d.vx, d.vy, d.vz};
    for (int c = 0; c < 9; ++c) a.rx[c * P + p] = src[c][p];
    for (int c = 0; c < 3; ++c) {
        double v;
        if (d.fp64) v = ((const double *)d.f)[c * P + p] + ((const double *)d.flr)[c * P + p];
        else v = (double)(long long)(d.f[c * P + p] + d.flr[c * P + p]) * (1.0 / kFixScale);
        a.rf[c * P + p] = v;
    }
    if (blockIdx.x == 0)
        for (int r = threadIdx.x; r < d.R; r += blockDim.x) a.rlr[r] = d.rs[r].lr_now;
}

// nine packed host-order arrays (replicas end to end, n values each) <-> nine
// component-major device arrays of P values (padding slots zero)
__global__ void __launch_bounds__(kBlock) k_adj_unpack(Dev d, double *dst, const double *stage, int N, unsigned mask)
{
    const int p = blockIdx.x * kBlock + threadIdx.x;
    const RepParams *R = d.rp + d.blk_rep[blockIdx.x];
    const int i = p - R->p0;
    for (int c = 0; c < 9; ++c)
        dst[(size_t)c * d.P + p] = (i < R->n && ((mask >> c) & 1u)) ? stage[(size_t)c * N + R->pk0 + i] : 0.0;
}

__global__ void __launch_bounds__(kBlock) k_adj_pack(Dev d, const double *src, double *stage, int N)
{
    const int p = blockIdx.x * kBlock + threadIdx.x;
    const RepParams *R = d.rp + d.blk_rep[blockIdx.x];
    const int i = p - R->p0;
    if (i >= R->n) return;
    for (int c = 0; c < 9; ++c) stage[(size_t)c * N + R->pk0 + i] = src[(size_t)c * d.P + p];
}

}  // namespace

void launch_adj_pair(const Dev &d, const AdjDev &a, cudaStream_t s, bool lr, const double *tan, int mode)
{
    // the Jacobian products of a mixed-precision engine in FP32 duals (its forward
    // pair math is FP32); dU/dtheta and FP64 engines in FP64 duals
    if (mode == 1 && !d.fp64) {
        if (lr) k_adj_pair<true, float><<<d.nblk, kBlock, 0, s>>>(d, a, tan, mode);
        else k_adj_pair<false, float><<<d.nblk, kBlock, 0, s>>>(d, a, tan, mode);
    } else {
        if (lr) k_adj_pair<true, double><<<d.nblk, kBlock, 0, s>>>(d, a, tan, mode);
        else k_adj_pair<false, double><<<d.nblk, kBlock, 0, s>>>(d, a, tan, mode);
    }
}

void launch_adj_topo(const Dev &d, const AdjDev &a, cudaStream_t s, const double *tan, int mode)
{
    const int n = d.nbt + d.nst3 + d.nst2 + a.nhb;
    if (n <= 0) return;
    const int nb = (n + kAdjTopoThreads - 1) / kAdjTopoThreads;
    if (mode == 1 && !d.fp64) k_adj_topo<float><<<nb, kAdjTopoThreads, 0, s>>>(d, a, tan, mode);
    else k_adj_topo<double><<<nb, kAdjTopoThreads, 0, s>>>(d, a, tan, mode);
}

void launch_adj_step(const Dev &d, const AdjDev &a, cudaStream_t s)
{
    cudaMemsetAsync(a.cen, 0, sizeof(double) * 3 * d.R, s);
    k_adj_center<<<d.nblk, kBlock, 0, s>>>(d, a);
    k_adj_move<<<d.nblk, kBlock, 0, s>>>(d, a);
    launch_adj_pair(d, a, s, false, a.lamf, 1);
    launch_adj_topo(d, a, s, a.lamf, 1);
    launch_adj_pair(d, a, s, true, a.mu, 1);
    k_adj_finish<<<d.nblk, kBlock, 0, s>>>(d, a);
}

void launch_adj_record(const Dev &d, const AdjDev &a, cudaStream_t s) { k_adj_record<<<d.nblk, kBlock, 0, s>>>(d, a); }

void launch_adj_unpack(const Dev &d, cudaStream_t s, double *dst, const double *stage, int n, unsigned mask)
{
    k_adj_unpack<<<d.nblk, kBlock, 0, s>>>(d, dst, stage, n, mask);
}

void launch_adj_pack(const Dev &d, cudaStream_t s, const double *src, double *stage, int n)
{
    k_adj_pack<<<d.nblk, kBlock, 0, s>>>(d, src, stage, n);
}

}  // namespace tis
