// CUDA kernels of the TIS-RNA Langevin step for sm_103a.
//
// One step of every replica (E: = src/16SCD_Mg_Cl_K_COPY_fast.cpp):
//   k_pair_sr     SR_interactions_lists      E:1783-1847   per particle, full neighbour list
//   k_pair_lr     LR_interactions_lists      E:1851-1907   every lr_interval steps or after a rebuild
//   k_bonded_stack polymer_constraints      E:2354-2520   one thread per term, all replicas
//                  stacking_interactions    E:1911-2141
//   k_hbond       hydrogen_bonds_interactions E:2145-2350  one block per replica:
//                 energies, valence-limited MC, forces; full_forces' Gaussians E:2590-2611
//   k_integrate   full_forces (application) + move_rigid_units + leap_frog_move_atom + adjust_box
//                                             E:2612-2732, E:570-642; its last block per
//                 replica runs check_shifts      E:1741-1776
//   rebuild       populate_lists + separate_in_cells E:1461-1737, gated per replica
#include <cstdio>

#include "tis_kernels.cuh"

namespace tis {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// Programmatic dependent launch: the kernels of a step's sequential chain are
// launched so that their blocks may be scheduled while the previous kernel on
// the stream drains; each waits here, before its first global access, until that
// kernel has finished and its writes are visible (a no-op for a normal launch).
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ---------------------------------------------------------------------------
// position and force accessors
// ---------------------------------------------------------------------------
template <bool D>
struct Pos;

template <>
struct Pos<false> {  // exact int32 differences -> FP32
    const int4 *q;
    float sx, sy, sz;
    __device__ V3<float> vec(int a, int b) const  // position(b) - position(a)
    {
        int4 qa = q[a], qb = q[b];
        return {(float)(int)((unsigned)qb.x - (unsigned)qa.x) * sx, (float)(int)((unsigned)qb.y - (unsigned)qa.y) * sy,
                (float)(int)((unsigned)qb.z - (unsigned)qa.z) * sz};
    }
};

template <>
struct Pos<true> {  // FP64 raw differences, no image (as the reference's bonded terms)
    const double *x, *y, *z;
    __device__ V3<double> vec(int a, int b) const { return {x[b] - x[a], y[b] - y[a], z[b] - z[a]}; }
};

template <bool D>
struct Acc;

template <>
struct Acc<false> {
    unsigned long long *f;
    int P;
    int err;
    __device__ void add(int i, V3<float> v)
    {
        atomic_add_fix(f + i, to_fix(v.x, err));
        atomic_add_fix(f + P + i, to_fix(v.y, err));
        atomic_add_fix(f + 2 * P + i, to_fix(v.z, err));
    }
};

template <>
struct Acc<true> {
    double *f;
    int P;
    int err;
    __device__ void add(int i, V3<double> v)
    {
        atomicAdd(f + i, v.x);
        atomicAdd(f + P + i, v.y);
        atomicAdd(f + 2 * P + i, v.z);
    }
};

template <bool D>
using Real = typename std::conditional<D, double, float>::type;

template <bool D>
__device__ inline Pos<D> make_pos(const Dev &d, const RepParams *R);
template <>
__device__ inline Pos<false> make_pos<false>(const Dev &d, const RepParams *R)
{
    return Pos<false>{d.q, R->qstep[0], R->qstep[1], R->qstep[2]};
}
template <>
__device__ inline Pos<true> make_pos<true>(const Dev &d, const RepParams *)
{
    return Pos<true>{d.x, d.y, d.z};
}

__device__ inline float atan2_(float a, float b) { return atan2f(a, b); }
__device__ inline double atan2_(double a, double b) { return atan2(a, b); }
__device__ inline float exp_(float v) { return expf(v); }
__device__ inline double exp_(double v) { return exp(v); }
__device__ inline float sqrt_(float v) { return sqrtf(v); }
__device__ inline double sqrt_(double v) { return sqrt(v); }
__device__ inline float rsqrt_(float v) { return 1.0f / sqrtf(v); }
__device__ inline double rsqrt_(double v) { return 1.0 / sqrt(v); }

// ---------------------------------------------------------------------------
// geometry and restraint forces (E:924-1454)
// ---------------------------------------------------------------------------
// valence_angle (E:986-1027): the angle at i2, as atan2(|a x b|, a.b), which
// equals the reference's acos(a.b / |a||b|) and stays accurate near 0 and pi.
template <bool D>
__device__ Real<D> angle_of(const Pos<D> &P, int i1, int i2, int i3)
{
    using R = Real<D>;
    V3<R> a = P.vec(i2, i1), b = P.vec(i2, i3);
    V3<R> w = cross(a, b);
    return atan2_(sqrt_(dot(w, w)), dot(a, b));
}

// dihedral_angle (E:1255-1302)
template <bool D>
__device__ Real<D> dihedral_of(const Pos<D> &P, int i1, int i2, int i3, int i4)
{
    using R = Real<D>;
    V3<R> v1 = P.vec(i1, i2), v2 = P.vec(i2, i3), v3 = P.vec(i3, i4);
    V3<R> m = cross(v1, v2), n = cross(v2, v3);
    return atan2_(dot(v1, n) * sqrt_(dot(v2, v2)), dot(m, n));
}

// harmonic bond k0 (r0 - r)^2 (bead_bond_force / stacking_bond_force, E:924-982)
template <bool D>
__device__ void bond_force(const Pos<D> &P, Acc<D> &A, int i1, int i2, Real<D> k0, Real<D> r0)
{
    using R = Real<D>;
    V3<R> v = P.vec(i1, i2);
    R r = sqrt_(dot(v, v));
    R t = R(2) * k0 * (r0 - r) / r;
    V3<R> g = t * v;
    A.add(i1, R(-1) * g);
    A.add(i2, g);
}

// harmonic angle k0 (theta0 - theta)^2 at i2 (bead_valence_force E:1031-1134;
// clamp = stacking_valence_force E:1138-1251, no force once cos theta < -0.99995).
// The reference writes the force as s d(cos theta)/dx with s = -2 k0 (theta0 -
// theta) / sin theta; this is the same vector, 2 k0 (theta0 - theta) d theta/dx,
// with d theta/dx1 = a x w / (|a|^2 |w|), d theta/dx3 = -b x w / (|b|^2 |w|),
// w = a x b, which keeps FP32 accurate where sin theta is small.
template <bool D>
__device__ void angle_force(const Pos<D> &P, Acc<D> &A, int i1, int i2, int i3, Real<D> k0, Real<D> th0, bool clamp)
{
    using R = Real<D>;
    V3<R> a = P.vec(i2, i1), b = P.vec(i2, i3);
    const R aa = dot(a, a), bb = dot(b, b), ab = dot(a, b);
    if (clamp && ab * rsqrt_(aa * bb) < R(-0.99995)) return;  // theta = pi, no force
    const V3<R> w = cross(a, b);
    const R ww = sqrt_(dot(w, w));
    if (ww == R(0)) return;
    const R th = atan2_(ww, ab);
    const R s = R(2) * k0 * (th0 - th) / ww;
    const V3<R> g1 = (s / aa) * cross(a, w);
    const V3<R> g3 = (-s / bb) * cross(b, w);
    A.add(i1, g1);
    A.add(i2, R(-1) * (g1 + g3));
    A.add(i3, g3);
}

// harmonic dihedral k0 (psi0 - psi)^2 (stacking_dihedral_force, E:1306-1454).
// The reference's s d(cos psi)/dx with s = -2 k0 (psi0 - psi) / sin psi equals
// 2 k0 (psi0 - psi) d psi/dx; here d psi/dx uses the cross-product form
// d psi/dx1 = -|v2| m / |m|^2, d psi/dx4 = |v2| n / |n|^2,
// d psi/dx2 = -(1 + v1.v2/|v2|^2) d psi/dx1 + (v3.v2/|v2|^2) d psi/dx4,
// which has no 1/sin psi and so no FP32 cancellation at planar (psi ~ 0, pi) geometry.
template <bool D>
__device__ void dihedral_force(const Pos<D> &P, Acc<D> &A, int i1, int i2, int i3, int i4, Real<D> k0,
                               Real<D> psi0)
{
    using R = Real<D>;
    const V3<R> v1 = P.vec(i1, i2), v2 = P.vec(i2, i3), v3 = P.vec(i3, i4);
    const V3<R> m = cross(v1, v2), n = cross(v2, v3);
    const R mm = dot(m, m), nn = dot(n, n), v22 = dot(v2, v2);
    if (mm == R(0) || nn == R(0)) return;
    const R l2 = sqrt_(v22);
    const R psi = atan2_(dot(v1, n) * l2, dot(m, n));
    const R c = R(2) * k0 * (psi0 - psi);
    const V3<R> g1 = (-c * l2 / mm) * m;
    const V3<R> g4 = (c * l2 / nn) * n;
    const R p = dot(v1, v2) / v22, q = dot(v3, v2) / v22;
    const V3<R> g2 = (R(-1) - p) * g1 + q * g4;
    A.add(i1, g1);
    A.add(i2, g2);
    A.add(i3, R(-1) * (g1 + g2 + g4));
    A.add(i4, g4);
}

// native dihedral imaged to within pi of the current one (E:1999-2019): branch -1/0/+1
template <class R>
__device__ inline int psi_branch(R psi, R nat)
{
    const R pi = R(3.14159265358979323846);
    if (fabs(psi - nat) <= pi) return 0;
    return (psi - nat > pi) ? 1 : -1;
}

template <class R>
__device__ inline R psi_shift(R nat, int br)
{
    return nat + R(2.0 * 3.14159265358979323846) * R(br);
}

// six-term native-geometry restraint (E:1983-2056, E:2177-2231, E:2319-2349)
template <bool D>
__device__ Real<D> six_q(const Pos<D> &P, const int *k, const double *nat, Real<D> rdev, Real<D> init, int &code)
{
    using R = Real<D>;
    R t1 = angle_of<D>(P, k[0], k[1], k[4]);
    R t2 = angle_of<D>(P, k[3], k[4], k[1]);
    R p0 = dihedral_of<D>(P, k[0], k[1], k[4], k[3]);
    R p1 = dihedral_of<D>(P, k[4], k[1], k[0], k[2]);
    R p2 = dihedral_of<D>(P, k[1], k[4], k[3], k[5]);
    int b0 = psi_branch<R>(p0, (R)nat[3]), b1 = psi_branch<R>(p1, (R)nat[4]), b2 = psi_branch<R>(p2, (R)nat[5]);
    code = (b0 + 1) + 3 * (b1 + 1) + 9 * (b2 + 1);
    R d0 = p0 - psi_shift<R>((R)nat[3], b0), d1 = p1 - psi_shift<R>((R)nat[4], b1), d2 = p2 - psi_shift<R>((R)nat[5], b2);
    R q = init + R(5) * rdev * rdev;
    q += R(1.5) * (t1 - (R)nat[1]) * (t1 - (R)nat[1]);
    q += R(1.5) * (t2 - (R)nat[2]) * (t2 - (R)nat[2]);
    q += R(0.15) * d0 * d0;
    q += R(0.15) * d1 * d1;
    q += R(0.15) * d2 * d2;
    return q;
}

template <bool D>
__device__ void six_force(const Pos<D> &P, Acc<D> &A, const int *k, const double *nat, int code, Real<D> w)
{
    using R = Real<D>;
    int b0 = code % 3 - 1, b1 = (code / 3) % 3 - 1, b2 = code / 9 - 1;
    bond_force<D>(P, A, k[1], k[4], R(5) * w, (R)nat[0]);
    angle_force<D>(P, A, k[0], k[1], k[4], R(1.5) * w, (R)nat[1], true);
    angle_force<D>(P, A, k[3], k[4], k[1], R(1.5) * w, (R)nat[2], true);
    dihedral_force<D>(P, A, k[0], k[1], k[4], k[3], R(0.15) * w, psi_shift<R>((R)nat[3], b0));
    dihedral_force<D>(P, A, k[4], k[1], k[0], k[2], R(0.15) * w, psi_shift<R>((R)nat[4], b1));
    dihedral_force<D>(P, A, k[1], k[4], k[3], k[5], R(0.15) * w, psi_shift<R>((R)nat[5], b2));
}

// Term s of the six-term restraint (0: the central distance, from rdev; 1-2: the
// angles; 3-5: the dihedrals, with the imaging branch of each in br): its weighted
// squared deviation, as six_q adds it.
template <bool D>
__device__ inline Real<D> six_term(const Pos<D> &P, const int *k, const double *nat, int s, Real<D> rdev, int &br)
{
    using R = Real<D>;
    br = 0;
    if (s == 0) return R(5) * rdev * rdev;
    if (s <= 2) {
        const R t = s == 1 ? angle_of<D>(P, k[0], k[1], k[4]) : angle_of<D>(P, k[3], k[4], k[1]);
        const R n = (R)nat[s];
        return R(1.5) * (t - n) * (t - n);
    }
    R p;
    if (s == 3) p = dihedral_of<D>(P, k[0], k[1], k[4], k[3]);
    else if (s == 4) p = dihedral_of<D>(P, k[4], k[1], k[0], k[2]);
    else p = dihedral_of<D>(P, k[1], k[4], k[3], k[5]);
    br = psi_branch<R>(p, (R)nat[s]);
    const R dd = p - psi_shift<R>((R)nat[s], br);
    return R(0.15) * dd * dd;
}

// force of term s of the six-term restraint (six_force's six calls, one at a time)
template <bool D>
__device__ inline void six_force_term(const Pos<D> &P, Acc<D> &A, const int *k, const double *nat, int code,
                                      Real<D> w, int s)
{
    using R = Real<D>;
    if (s == 0) bond_force<D>(P, A, k[1], k[4], R(5) * w, (R)nat[0]);
    else if (s == 1) angle_force<D>(P, A, k[0], k[1], k[4], R(1.5) * w, (R)nat[1], true);
    else if (s == 2) angle_force<D>(P, A, k[3], k[4], k[1], R(1.5) * w, (R)nat[2], true);
    else if (s == 3) dihedral_force<D>(P, A, k[0], k[1], k[4], k[3], R(0.15) * w, psi_shift<R>((R)nat[3], code % 3 - 1));
    else if (s == 4)
        dihedral_force<D>(P, A, k[4], k[1], k[0], k[2], R(0.15) * w, psi_shift<R>((R)nat[4], (code / 3) % 3 - 1));
    else dihedral_force<D>(P, A, k[1], k[4], k[3], k[5], R(0.15) * w, psi_shift<R>((R)nat[5], code / 9 - 1));
}

template <bool D>
__device__ inline Real<D> distance(const Pos<D> &P, int a, int b)
{
    V3<Real<D>> v = P.vec(a, b);
    return sqrt_(dot(v, v));
}

// ---------------------------------------------------------------------------
// exact FP64 pair distance with the reference's image rule (CC_vector, E:674-683)
// ---------------------------------------------------------------------------
__device__ inline double exact_r2(const Dev &d, const RepParams *R, int i, int j)
{
    double a = __dsub_rn(d.x[i], d.x[j]);
    double b = __dsub_rn(d.y[i], d.y[j]);
    double c = __dsub_rn(d.z[i], d.z[j]);
    if (a > R->hbox[0]) a = __dsub_rn(a, R->box[0]);
    if (a < -R->hbox[0]) a = __dadd_rn(a, R->box[0]);
    if (b > R->hbox[1]) b = __dsub_rn(b, R->box[1]);
    if (b < -R->hbox[1]) b = __dadd_rn(b, R->box[1]);
    if (c > R->hbox[2]) c = __dsub_rn(c, R->box[2]);
    if (c < -R->hbox[2]) c = __dadd_rn(c, R->box[2]);
    return __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
}

__device__ inline void exact_vec(const Dev &d, const RepParams *R, int i, int j, double v[3])
{
    v[0] = d.x[i] - d.x[j];
    v[1] = d.y[i] - d.y[j];
    v[2] = d.z[i] - d.z[j];
    for (int k = 0; k < 3; ++k) {
        if (v[k] > R->hbox[k]) v[k] = v[k] - R->box[k];
        if (v[k] < -R->hbox[k]) v[k] = v[k] + R->box[k];
    }
}

__device__ inline bool is_charged(int kind) { return kind != 1 && kind != 2; }

// Relative half-width of the band around a threshold inside which the FP32
// squared distance cannot decide a comparison and the exact FP64 one is used.
constexpr float kBand = 1.0e-5f;

// ---------------------------------------------------------------------------
// quantisation: fixed-point copy of the FP64 positions
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_quantize(Dev d)
{
    int p = blockIdx.x * kBlock + threadIdx.x;
    const RepParams *R = d.rp + d.blk_rep[blockIdx.x];
    int4 q = d.q[p];
    q.x = (int)(unsigned)(long long)floor(d.x[p] * R->qinv[0]);
    q.y = (int)(unsigned)(long long)floor(d.y[p] * R->qinv[1]);
    q.z = (int)(unsigned)(long long)floor(d.z[p] * R->qinv[2]);
    d.q[p] = q;
}

// packed (unpadded, replicas end to end) state <-> the padded device arrays; N is
// the group's particle count, stage holds the nine arrays of N values each
__global__ void __launch_bounds__(kBlock) k_put_state(Dev d, const double *stage, int N)
{
    const int p = blockIdx.x * kBlock + threadIdx.x;
    const RepParams *R = d.rp + d.blk_rep[blockIdx.x];
    const int i = p - R->p0;
    if (i >= R->n) return;
    double *dst[9] = {d.x, d.y, d.z, d.xo, d.yo, d.zo, d.vx, d.vy, d.vz};
    for (int c = 0; c < 9; ++c) dst[c][p] = stage[(size_t)c * N + R->pk0 + i];
    int4 q = d.q[p];
    q.x = (int)(unsigned)(long long)floor(d.x[p] * R->qinv[0]);
    q.y = (int)(unsigned)(long long)floor(d.y[p] * R->qinv[1]);
    q.z = (int)(unsigned)(long long)floor(d.z[p] * R->qinv[2]);
    d.q[p] = q;
}

__global__ void __launch_bounds__(kBlock) k_get_state(Dev d, double *stage, int N, unsigned mask)
{
    const int p = blockIdx.x * kBlock + threadIdx.x;
    const RepParams *R = d.rp + d.blk_rep[blockIdx.x];
    const int i = p - R->p0;
    if (i >= R->n) return;
    const double *src[9] = {d.x, d.y, d.z, d.xo, d.yo, d.zo, d.vx, d.vy, d.vz};
    for (int c = 0; c < 9; ++c)
        if ((mask >> c) & 1u) stage[(size_t)c * N + R->pk0 + i] = src[c][p];
}

// ---------------------------------------------------------------------------
// pair forces over the full (both-direction) neighbour lists
// ---------------------------------------------------------------------------
// Loads of data that the fused step kernel rewrites while it runs (positions,
// lists) go through L2, the coherent path; the step's separate kernels read them
// through the read-only path.
template <bool CO, class T>
__device__ __forceinline__ T ld_in(const T *ptr)
{
    if (CO) return __ldcg(ptr);
    return __ldg(ptr);
}

// the replica's FP32 pair tables as the pair code reads them (shared memory copies)
struct PairTables {
    const float *dlj2, *dm, *flj, *qclb;
};

// The pair forces of particle p over its full list, by L threads (lane4 = its lane
// among them): slot k of the list goes to lane k % L; lane 0 adds the sum (LR: stores
// the held LR force).  err, e_lj, e_c accumulate per thread.
template <bool D, bool LR, bool EN, bool EX, int L, bool CO>
__device__ __forceinline__ void pair_particle(const Dev &d, const RepParams *R, int p, int lane4, const PairTables &tb,
                                              int &err, double &e_lj, double &e_c)
{
    const int P = d.P;
    const int4 qp = d.q[p];
    const int tp = qp.w & 0xff, kp = (qp.w >> 8) & 0xff, act = (qp.w >> 16) & 1;
    const bool chp = is_charged(kp);
    const int cnt = act ? (LR ? d.n_lr[p] : d.n_sr[p]) : 0;
    const int *nbr = LR ? d.nbr_lr : d.nbr_sr;
    if (!D) {
        long long ax = 0, ay = 0, az = 0;
        const float sx = R->qstep[0], sy = R->qstep[1], sz = R->qstep[2];
        const float rc2 = R->rc2f, lo = rc2 * (1.0f - kBand), hi = rc2 * (1.0f + kBand);
        const float kap = R->kappaf;
        for (int k = lane4; k < cnt; k += L) {
            const int raw = ld_in<CO>(nbr + nb_idx(k, p, P));
            const int j = raw & kIdxMask;
            const float ljw = EX ? (float)(1 - (raw >> kExclShift)) : 1.0f;
            const int4 qj = ld_in<CO>(d.q + j);
            const float dx = (float)(int)((unsigned)qp.x - (unsigned)qj.x) * sx;
            const float dy = (float)(int)((unsigned)qp.y - (unsigned)qj.y) * sy;
            const float dz = (float)(int)((unsigned)qp.z - (unsigned)qj.z) * sz;
            const float r2 = dx * dx + dy * dy + dz * dz;
            const int tj = qj.w & 0xff, kj = (qj.w >> 8) & 0xff;
            const int J = jn12(tp, tj);
            float F = 0.0f;
            if (!LR && ljw != 0.0f && r2 <= tb.dlj2[J]) {  // LJ_FORCE (E:801-821)
                const float rr = sqrtf(r2);
                const float dr = rr - tb.dm[J];
                const float s = 1.5852f / dr;
                const float s2 = s * s, s4 = s2 * s2, s8 = s4 * s4, s14 = s8 * s4 * s2;
                F = ljw * (tb.flj[J] * (s14 - s8) * dr / rr);
                if (EN) {
                    double e;
                    if ((double)r2 < R->d2min_d[J]) e = R->elj_d[J] * 1001.0;
                    else {
                        const float s6 = s4 * s2, s12 = s6 * s6;
                        e = (double)(R->elj[J] * (s12 - 2.0f * s6 + 1.0f));
                    }
                    e_lj += 0.5 * (double)ljw * e;
                }
            }
            if ((LR || (chp && is_charged(kj))) && r2 <= hi) {  // COULOMB_TRUNCATED_FORCE (E:841-855)
                bool in = r2 <= lo || exact_r2(d, R, p, j) <= R->rc2;
                if (in) {
                    const float rr = sqrtf(r2);
                    if (kap == 0.0f) {
                        F += tb.qclb[J] / (r2 * rr);
                        if (EN) e_c += 0.5 * (double)(tb.qclb[J] / rr);
                    } else {  // screened: U = C exp(-kappa r) / r, F / r = U (1 + kappa r) / r^2
                        const float kr = kap * rr, u = tb.qclb[J] * expf(-kr) / rr;
                        F += u * (1.0f + kr) / r2;
                        if (EN) e_c += 0.5 * (double)u;
                    }
                }
            }
            if (F != 0.0f) {
                ax += to_fix(F * dx, err);
                ay += to_fix(F * dy, err);
                az += to_fix(F * dz, err);
            }
        }
        for (int o = 1; o < L; o <<= 1) {
            ax += __shfl_xor_sync(kFull, ax, o);
            ay += __shfl_xor_sync(kFull, ay, o);
            az += __shfl_xor_sync(kFull, az, o);
        }
        if (lane4 == 0) {
            if (LR) {  // the LR force is kept for the MTS interval: overwrite
                d.flr[p] = (unsigned long long)ax;
                d.flr[P + p] = (unsigned long long)ay;
                d.flr[2 * P + p] = (unsigned long long)az;
            } else if (act) {  // other force kernels run concurrently: accumulate
                atomic_add_fix(d.f + p, ax);
                atomic_add_fix(d.f + P + p, ay);
                atomic_add_fix(d.f + 2 * P + p, az);
            }
        }
    } else {
        double ax = 0, ay = 0, az = 0;
        for (int k = lane4; k < cnt; k += L) {
            const int raw = ld_in<CO>(nbr + nb_idx(k, p, P));
            const int j = raw & kIdxMask;
            const double ljw = EX ? (double)(1 - (raw >> kExclShift)) : 1.0;
            const int tj = d.q[j].w & 0xff, kj = (d.q[j].w >> 8) & 0xff;
            const int J = jn12(tp, tj);
            double v[3];
            exact_vec(d, R, p, j, v);
            const double r2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            double F = 0.0;
            if (!LR && ljw != 0.0 && r2 <= R->dlj2_d[J]) {
                const double rr = sqrt(r2);
                const double dr = rr + kSig0 - R->dlj_d[J];
                const double s = kSig0 / dr;
                const double s2 = s * s, s4 = s2 * s2, s8 = s4 * s4, s14 = s8 * s4 * s2;
                F = ljw * (R->flj_d[J] * (s14 - s8) * dr / rr);
                if (EN) {
                    double e;
                    if (r2 < R->d2min_d[J]) e = R->elj_d[J] * 1001.0;
                    else {
                        const double s6 = s4 * s2, s12 = s6 * s6;
                        e = R->elj_d[J] * (s12 - 2.0 * s6 + 1.0);
                    }
                    e_lj += 0.5 * ljw * e;
                }
            }
            if ((LR || (chp && is_charged(kj))) && r2 <= R->rc2) {
                const double rr = sqrt(r2);
                if (R->kappa == 0.0) {
                    F += R->qclb_d[J] / (rr * r2);
                    if (EN) e_c += 0.5 * R->qclb_d[J] / rr;
                } else {
                    const double kr = R->kappa * rr, u = R->qclb_d[J] * exp(-kr) / rr;
                    F += u * (1.0 + kr) / r2;
                    if (EN) e_c += 0.5 * u;
                }
            }
            ax += v[0] * F;
            ay += v[1] * F;
            az += v[2] * F;
        }
        for (int o = 1; o < L; o <<= 1) {
            ax += __shfl_xor_sync(kFull, ax, o);
            ay += __shfl_xor_sync(kFull, ay, o);
            az += __shfl_xor_sync(kFull, az, o);
        }
        if (lane4 == 0) {
            if (LR) {
                double *out = (double *)d.flr;
                out[p] = ax;
                out[P + p] = ay;
                out[2 * P + p] = az;
            } else if (act) {
                double *out = (double *)d.f;
                atomicAdd(out + p, ax);
                atomicAdd(out + P + p, ay);
                atomicAdd(out + 2 * P + p, az);
            }
        }
    }
}

// Particle block b (kBlock particles) by T threads, L per particle: slot k of a
// particle's list goes to its thread k % L; the block's particles in kBlock L / T passes.
template <bool D, bool LR, bool EN, bool EX, int L, int T>
__device__ void pair_block(const Dev &d, int b, int force_all)
{
    const int r = d.blk_rep[b];
    const RepParams *R = d.rp + r;
    if (LR && !force_all && !d.rs[r].lr_now) return;
    __shared__ float s_dlj2[46], s_dm[46], s_flj[46], s_qclb[46];
    if (!D) {
        for (int t = threadIdx.x; t < 46; t += blockDim.x) {
            s_dlj2[t] = R->dlj2[t];
            s_dm[t] = R->dm[t];
            s_flj[t] = R->flj[t];
            s_qclb[t] = R->qclb[t];
        }
        __syncthreads();
    }
    const PairTables tb{s_dlj2, s_dm, s_flj, s_qclb};
    const int lane4 = threadIdx.x & (L - 1);
    int err = 0;
    double e_lj = 0, e_c = 0;
    constexpr int kPasses = kBlock * L / T;
#pragma unroll
    for (int pass = 0; pass < kPasses; ++pass) {
        const int p = b * kBlock + pass * (T / L) + (int)threadIdx.x / L;
        pair_particle<D, LR, EN, EX, L, false>(d, R, p, lane4, tb, err, e_lj, e_c);
    }
    if (EN) {
        if (!LR) atomicAdd(d.eterm + r * kNE + 0, e_lj);
        atomicAdd(d.eterm + r * kNE + (LR ? 2 : 1), e_c);
    }
    if (err) atomicOr(&d.rs[r].err, err);
}

template <bool D, bool LR, bool EN, bool EX, int L, int T>
__global__ void __launch_bounds__(T) k_pair(Dev d, int force_all)
{
    pair_block<D, LR, EN, EX, L, T>(d, blockIdx.x, force_all);
}

// ---------------------------------------------------------------------------
// block reductions
// ---------------------------------------------------------------------------
// barriers of the threads that run a block-level part: the whole CTA, or warps
// 0 .. n/32-1 of it on a named barrier (the fused step kernel's H-bond warps)
struct CtaBar {
    __device__ void operator()() const { __syncthreads(); }
};
struct NamedBar {
    int id, n;
    __device__ void operator()() const { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
};

// sum of NV doubles over threads tid = 0 .. nthr-1 (a multiple of 32) into tid 0
template <int NV, class Bar>
__device__ void block_sum_t(double (&v)[NV], double *smem /* NV * 32 */, int tid, int nthr, Bar bar)
{
    const int lane = tid & 31, w = tid >> 5, nw = (nthr + 31) >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i)
        for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_down_sync(kFull, v[i], o);
    bar();
    if (lane == 0)
        for (int i = 0; i < NV; ++i) smem[i * 32 + w] = v[i];
    bar();
    if (w == 0) {
        for (int i = 0; i < NV; ++i) {
            double t = lane < nw ? smem[i * 32 + lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(kFull, t, o);
            v[i] = t;
        }
    }
    bar();
}

template <int NV>
__device__ void block_sum(double (&v)[NV], double *smem /* NV * 32 */)
{
    block_sum_t<NV>(v, smem, (int)threadIdx.x, (int)blockDim.x, CtaBar{});
}

// ---------------------------------------------------------------------------
// integrator: noise application, leap-frog, recentring, ion wrap, skin check
// ---------------------------------------------------------------------------
template <bool D>
__device__ inline double total_force(const Dev &d, int p, int c)
{
    if (D) {
        const double *f = (const double *)d.f, *fl = (const double *)d.flr;
        return __ldcg(f + c * d.P + p) + __ldcg(fl + c * d.P + p);
    }
    const long long t = (long long)(__ldcg(d.f + c * d.P + p) + __ldcg(d.flr + c * d.P + p));
    return (double)t * (1.0 / kFixScale);
}

// leap_frog_move_atom (E:570-642) with the noise of full_forces (E:2612-2622).
// FP64 mode follows the reference's operation order.  Mixed mode evaluates the
// same update v' = K1 v + K2 (f + g sigma) as K1 v + (K2 2^-32) f_fix + (K2 sigma) g
// with fused multiply-adds, and x' = x + (x - x_old) + (v' - v) h; the velocity
// cap m v'^2 / (300 T) > 1 uses the precomputed m / (300 T) in both modes.
template <bool D>
__device__ inline void leap_frog(const Dev &d, const RepParams *R, int r, int p, double xn[3], double vn[3])
{
    const int t = d.q[p].w & 0xff;
    const double v0[3] = {d.vx[p], d.vy[p], d.vz[p]};
    const double x0[3] = {d.x[p], d.y[p], d.z[p]};
    const double o0[3] = {d.xo[p], d.yo[p], d.zo[p]};
    const int k = (p - R->p0 + 1) % 1000;
    const double *g = d.gnoise + r * kNoise;
    if (D) {
        double f[3] = {total_force<D>(d, p, 0), total_force<D>(d, p, 1), total_force<D>(d, p, 2)};
        if (d.noise == 0) {
            const double sg = R->sigma[t];
            for (int c = 0; c < 3; ++c) f[c] = __dadd_rn(f[c], __dmul_rn(g[k + 1000 * c], sg));
        }
        for (int c = 0; c < 3; ++c) vn[c] = __dadd_rn(__dmul_rn(R->k1[t], v0[c]), __dmul_rn(R->k2[t], f[c]));
    } else {
        const double k1 = R->k1[t], kf = R->k2fix[t], kg = d.noise == 0 ? R->k2sig[t] : 0.0;
        for (int c = 0; c < 3; ++c) {
            const long long fx = (long long)(__ldcg(d.f + c * d.P + p) + __ldcg(d.flr + c * d.P + p));
            vn[c] = fma(kg, g[k + 1000 * c], fma(kf, (double)fx, k1 * v0[c]));
        }
    }
    double vsq = R->vcap[t] * (vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2]);
    if (vsq > 1.0) {
        vsq = 1.0 / sqrt(vsq);
        for (int c = 0; c < 3; ++c) vn[c] *= vsq;
    }
    if (D) {
        for (int c = 0; c < 3; ++c)
            xn[c] = __dadd_rn(__dsub_rn(__dmul_rn(2.0, x0[c]), o0[c]), __dmul_rn(__dsub_rn(vn[c], v0[c]), R->h));
    } else {
        for (int c = 0; c < 3; ++c) xn[c] = fma(vn[c] - v0[c], R->h, x0[c] + (x0[c] - o0[c]));
    }
}

// full_forces' Gaussians (E:2594-2606) of one replica from draw c0 on, by the
// threads of one block
template <bool D>
__device__ void gen_noise(const Dev &d, int r, unsigned long long c0, int tid, int nthr)
{
    const RepParams *R = d.rp + r;
    if (d.noise != 0) return;
    for (int t = tid; t < kNoise / 2; t += nthr) {
        const uint32_t v1 = rand_value(R->seed, c0 + 2 * t);
        const uint32_t v2 = rand_value(R->seed, c0 + 2 * t + 1);
        if (D) {  // Box-Muller as the reference forms it (E:2598-2606), in FP64
            const double a = sqrt(-2.0 * log(u31_ratio(v1)));
            const double b = 2.0 * 3.14159265358979323846 * u31_ratio(v2);
            double sn, cs;
            sincos(b, &sn, &cs);
            d.gnoise[r * kNoise + 2 * t] = a * cs;
            d.gnoise[r * kNoise + 2 * t + 1] = a * sn;
        } else {  // FP32 Box-Muller, radius accurate over the whole uniform range
            const float a = bm_radius(v1);
            float sn, cs;
            sincospif(2.0f * ((float)v2 * (1.0f / 2147483647.0f)), &sn, &cs);
            d.gnoise[r * kNoise + 2 * t] = (double)(a * cs);
            d.gnoise[r * kNoise + 2 * t + 1] = (double)(a * sn);
        }
    }
}

// the step's Gaussians alone (the drop-in full_forces call), one block per replica;
// the reference draws them even when the noise amplitude is zero
template <bool D>
__global__ void k_noise(Dev d)
{
    const int r = blockIdx.x;
    const unsigned long long c0 = d.rs[r].ctr;
    gen_noise<D>(d, r, c0, (int)threadIdx.x, (int)blockDim.x);
    __syncthreads();
    if (threadIdx.x == 0) d.rs[r].ctr = c0 + kNoise;
}

// ---------------------------------------------------------------------------
// bonded terms and stacks of every replica, one thread per term
// ---------------------------------------------------------------------------
constexpr int kTopoThreads = 256;

// LJ force of an excluded (bonded) pair, as reduce_forces subtracts it (E:880-897)
template <bool D, bool EN>
__device__ void exclusion_lj(const Dev &d, const RepParams *R, const Pos<D> &P, Acc<D> &A, int a, int ex,
                             double &e_excl)
{
    using Rl = Real<D>;
    const int ta = d.q[a].w & 0xff, tb = d.q[ex].w & 0xff;
    const int J = jn12(ta, tb);
    V3<Rl> v = P.vec(ex, a);  // x_a - x_ex, minimum image
    if (D) {
        double w[3];
        exact_vec(d, R, a, ex, w);
        v = V3<Rl>{(Rl)w[0], (Rl)w[1], (Rl)w[2]};
    }
    const Rl r2 = dot(v, v);
    if (!(r2 <= (Rl)(D ? R->dlj2_d[J] : R->dlj2[J]))) return;
    const Rl rr = sqrt_(r2);
    const Rl dr = D ? (Rl)(rr + kSig0 - R->dlj_d[J]) : (Rl)(rr - R->dm[J]);
    const Rl s = Rl(1.5852) / dr;
    const Rl s2 = s * s, s4 = s2 * s2, s8 = s4 * s4, s14 = s8 * s4 * s2;
    const Rl F = (Rl)(D ? R->flj_d[J] : R->flj[J]) * (s14 - s8) * dr / rr;
    if (EN) {
        double e;
        if ((double)r2 < R->d2min_d[J]) e = R->elj_d[J] * 1001.0;
        else {
            const Rl s6 = s4 * s2, s12 = s6 * s6;
            e = (double)((Rl)(D ? R->elj_d[J] : R->elj[J]) * (s12 - Rl(2) * s6 + Rl(1)));
        }
        e_excl -= e;
    }
    if (F != Rl(0)) {
        const V3<Rl> g = (Rl(-1) * F) * v;
        A.add(a, g);
        A.add(ex, Rl(-1) * g);
    }
}

// polymer_constraints (E:2354-2520), then stacking_interactions (E:1911-2141):
// items [0, nbt) are bonded terms, then tertiary stacks, then secondary stacks.
// A secondary stack is off this step when a tertiary stack sharing one of its
// sites (ST_EXCESS == 1) is within 10 A of its native distance (E:1960-1981);
// each secondary stack checks the few tertiary stacks that can do that.
// item t of the handle's bonded terms and stacks (above), by one thread
template <bool D, bool EN>
__device__ __forceinline__ void topo_item(const Dev &d, int t, int mask, int excl_in_list)
{
    using Rl = Real<D>;
    int r, kind;  // kind: 0 bonded, 1 tertiary, 2 secondary
    int item;
    if (t < d.nbt) { kind = 0; item = t; r = d.rep_of[d.bt_idx[t].x]; }
    else if (t < d.nbt + d.nst3) { kind = 1; item = t - d.nbt; r = d.rep_of[d.st3_idx[6 * item]]; }
    else if (t < d.nbt + d.nst3 + d.nst2) { kind = 2; item = t - d.nbt - d.nst3; r = d.rep_of[d.st2_idx[7 * item]]; }
    else return;
    if ((kind == 0 && !(mask & 4)) || (kind > 0 && !(mask & 8))) return;
    const RepParams *R = d.rp + r;
    const Pos<D> P = make_pos<D>(d, R);
    Acc<D> A;
    A.f = (decltype(A.f))d.f;
    A.P = d.P;
    A.err = 0;
    double e_excl = 0;
    if (kind == 0) {
        const int4 id = d.bt_idx[item];
        const double2 par = d.bt_par[item];
        const int ex = id.w == 0 ? id.y : id.z;  // excluded pair partner of id.x
        if (id.w == 0) bond_force<D>(P, A, id.x, id.y, (Rl)par.x, (Rl)par.y);
        else angle_force<D>(P, A, id.x, id.y, id.z, (Rl)par.x, (Rl)par.y, false);
        if (!excl_in_list || EN) exclusion_lj<D, EN>(d, R, P, A, id.x, ex, e_excl);
        if (EN) {
            double *e = d.eterm + r * kNE;
            if (id.w == 0) {
                const Rl rr = distance<D>(P, id.x, id.y);
                atomicAdd(e + 3, (double)((Rl)par.x * (rr - (Rl)par.y) * (rr - (Rl)par.y)));
            } else {
                const Rl th = angle_of<D>(P, id.x, id.y, id.z);
                atomicAdd(e + 4, (double)((Rl)par.x * (th - (Rl)par.y) * (th - (Rl)par.y)));
            }
            if (e_excl != 0) atomicAdd(e + 5, e_excl);
        }
    } else if (kind == 1) {
        const int *id = d.st3_idx + 6 * item;
        const double *nat = d.st3_nat + 6 * item;
        const Rl rdev = distance<D>(P, id[1], id[4]) - (Rl)nat[0];
        int code;
        const Rl Dn = six_q<D>(P, id, nat, rdev, Rl(1), code);
        const Rl E = (Rl)d.st3_E[item] / Dn;
        six_force<D>(P, A, id, nat, code, -E / Dn);
        d.st_energy[item] = (double)E;
        atomicAdd(EN ? d.eterm + r * kNE + 7 : &d.rs[r].e3st_acc, (double)E);
    } else {
        for (int u = d.st2_offby_off[item]; u < d.st2_offby_off[item + 1]; ++u) {
            const int k = d.st2_offby_idx[u];
            const int *tid = d.st3_idx + 6 * k;
            if (distance<D>(P, tid[1], tid[4]) - (Rl)d.st3_nat[6 * k] < Rl(10)) return;
        }
        const int *id = d.st2_idx + 7 * item;  // k_10 k00 k01 k10 k20 k21 k30
        const Rl rr = distance<D>(P, id[2], id[5]);
        const Rl p1 = dihedral_of<D>(P, id[0], id[1], id[3], id[4]);
        const Rl p2 = dihedral_of<D>(P, id[6], id[4], id[3], id[1]);
        const Rl p10 = psi_shift<Rl>(Rl(-2.58684), psi_branch<Rl>(p1, Rl(-2.58684)));
        const Rl p20 = psi_shift<Rl>(Rl(3.07135), psi_branch<Rl>(p2, Rl(3.07135)));
        const Rl r0 = (Rl)d.st2_r0[item];
        Rl Dn = Rl(1) + Rl(1.4) * (rr - r0) * (rr - r0);
        Dn += Rl(4) * (p1 - p10) * (p1 - p10);
        Dn += Rl(4) * (p2 - p20) * (p2 - p20);
        const Rl E = (Rl)d.st2_E[item] / Dn;
        const Rl w = -E / Dn;
        bond_force<D>(P, A, id[2], id[5], Rl(1.4) * w, r0);
        dihedral_force<D>(P, A, id[0], id[1], id[3], id[4], Rl(4) * w, p10);
        dihedral_force<D>(P, A, id[6], id[4], id[3], id[1], Rl(4) * w, p20);
        atomicAdd(EN ? d.eterm + r * kNE + 6 : &d.rs[r].e2st_acc, (double)E);
    }
    if (A.err) atomicOr(&d.rs[r].err, A.err);
}

template <bool D, bool EN>
__global__ void __launch_bounds__(kTopoThreads) k_bonded_stack(Dev d, int mask, int excl_in_list)
{
    topo_item<D, EN>(d, blockIdx.x * blockDim.x + threadIdx.x, mask, excl_in_list);
}

__device__ __forceinline__ unsigned long long global_ns_hb()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------
// hydrogen bonds of one replica per block: energies, the valence-limited Monte
// Carlo, forces; then (fused step) this step's Gaussians
// ---------------------------------------------------------------------------
// Working arrays of one replica's H-bonds, indexed by the replica's local bond
// and over-valence atom numbers: in shared memory when they fit (Dev::hb_smem),
// else in global scratch.  status starts as the list build left it (0: live,
// -1: out of range) and every live bond is back to 0 when the kernel ends, so
// the shared copy is never written back.
struct HbWork {
    double *en;    // energy of each live bond this step
    double *term;  // its six restraint terms (six per bond)
    int *st;       // status: 0 formed, 1 broken this step, -1 out of range
    int *code;     // imaging branch of its dihedrals
    int *br;       // the branches of its three dihedrals (three per bond)
    int *exc;      // excess valence of each over-valence atom
    int *al;       // over-valence atoms with positive excess (the reference's A list)
    int *kl;       // candidate bonds of the chosen atom (the reference's K list)
    const int *ca_off, *ca_idx;  // candidates of each over-valence atom: ca_idx[ca_off[i] ..]
    const int *hb_off, *hb_pos;  // over-valence atoms of each bond: hb_pos[hb_off[k] ..]
};

constexpr int kHbThreads = 512;

// rand() draws vbase .. vbase + 63 of a replica into v[], by 17 lanes of one warp
// (one Philox block of four draws each; the same words rand_value returns)
__device__ inline void fill_draws(uint32_t *v, unsigned long long seed, unsigned long long vbase, int lane)
{
    const unsigned long long b = (vbase >> 2) + (unsigned long long)lane;
    if (lane < 17) {
        uint32_t c[4] = {(uint32_t)b, (uint32_t)(b >> 32), 0u, 0u};
        philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        for (int w = 0; w < 4; ++w) {
            const long long idx = (long long)(4 * b + (unsigned long long)w) - (long long)vbase;
            if (idx >= 0 && idx < 64) {
                const uint32_t x = c[w] >> 1;
                v[idx] = x ? x : 1u;
            }
        }
    }
    __syncwarp();
}

// One block per replica.  The restraint energies and forces of the live bonds run
// as (chunk of 32 bonds, term) warp tasks, so that the lanes of a warp evaluate
// the same term; the Monte Carlo runs on one warp; then the step's Gaussians,
// drawn by the block while its warps finish the force tasks.
template <bool D, bool EN, class Bar>
__device__ __forceinline__ void hbond_block(const Dev &d, int r, int do_hb, int make_noise, int tid, int bd, Bar bar)
{
    using Rl = Real<D>;
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ uint32_t s_v[64];  // draws vbase .. vbase + 63 of the replica's rand() stream
    __shared__ unsigned long long s_ctr;
    __shared__ double s_red[2 * 32];
    const RepParams *R = d.rp + r;
    RepState *S = d.rs + r;
    const Pos<D> P = make_pos<D>(d, R);
    Acc<D> A;
    A.f = (decltype(A.f))d.f;
    A.P = d.P;
    A.err = 0;
    if (tid == 0) s_ctr = S->ctr;
    double e2hb = 0, e3hb = 0;
    const int hb0 = R->hb0, nhb = R->hb1 - R->hb0, ca0 = R->ca0, nca = R->ca1 - R->ca0;
    const int warp = tid >> 5, nwarp = bd >> 5, lane = tid & 31;
    // sub-phase times of the fused kernel's phase timer (tis_profile_fused), by tid 0
    unsigned long long *prof = (d.fprof && tid == 0) ? d.fprof + (size_t)r * kFusedPhases : nullptr;
    unsigned long long tlap = prof ? global_ns_hb() : 0ull;
    auto lap = [&](int k) {
        if (prof) {
            const unsigned long long t = global_ns_hb();
            atomicAdd(prof + k, t - tlap);
            tlap = t;
        }
    };
    HbWork w;
    const int nact = do_hb ? S->n_active : 0;
    bar();

    // ---- hydrogen_bonds_interactions (E:2145-2350) ----
    if (do_hb) {
        const int c_base = d.ca_coff[ca0], n_cidx = d.ca_coff[R->ca1] - c_base;
        const int h_base = d.hb_coff[hb0], n_cpos = d.hb_coff[R->hb1] - h_base;
        if (d.hb_smem) {
            const HbLayout L = hb_layout(d.hb_nmax, d.ca_nmax, d.k_nmax, d.cidx_max, d.cpos_max);
            w.en = (double *)(s_dyn + L.en);
            w.term = (double *)(s_dyn + L.term);
            w.st = (int *)(s_dyn + L.st);
            w.code = (int *)(s_dyn + L.code);
            w.br = (int *)(s_dyn + L.br);
            w.exc = (int *)(s_dyn + L.exc);
            w.al = (int *)(s_dyn + L.al);
            w.kl = (int *)(s_dyn + L.kl);
            int *cao = (int *)(s_dyn + L.ca_off), *cai = (int *)(s_dyn + L.ca_idx);
            int *hbo = (int *)(s_dyn + L.hb_off), *hbp = (int *)(s_dyn + L.hb_pos);
            for (int i = tid; i < nhb; i += bd) w.st[i] = d.hb_status[hb0 + i];
            for (int i = tid; i <= nca; i += bd) cao[i] = d.ca_coff[ca0 + i] - c_base;
            for (int i = tid; i < n_cidx; i += bd) cai[i] = d.ca_cidx[c_base + i];
            for (int i = tid; i <= nhb; i += bd) hbo[i] = d.hb_coff[hb0 + i] - h_base;
            for (int i = tid; i < n_cpos; i += bd) hbp[i] = d.hb_cpos[h_base + i];
            w.ca_off = cao; w.ca_idx = cai; w.hb_off = hbo; w.hb_pos = hbp;
        } else {
            w.en = d.hb_energy + hb0;
            w.term = d.hb_term + 6 * (size_t)hb0;
            w.st = d.hb_status + hb0;
            w.code = d.hb_code + hb0;
            w.br = d.hb_br + 3 * (size_t)hb0;
            w.exc = d.ca_exc + ca0;
            w.al = d.hb_A + ca0;
            w.kl = d.hb_K + R->kscr0;
            w.ca_off = d.ca_coff + ca0; w.ca_idx = d.ca_cidx;
            w.hb_off = d.hb_coff + hb0; w.hb_pos = d.hb_cpos;
        }
        for (int i = tid; i < nca; i += bd) w.exc[i] = d.hb_excess[d.ca_list[ca0 + i]];
        bar();
        // a live bond whose central distance strays more than 2 A from native breaks (E:2165-2175)
        for (int t = tid; t < nact; t += bd) {
            const int k = d.hb_active[hb0 + t], kl = k - hb0;
            const Rl rdev = distance<D>(P, d.hb_idx[6 * k + 1], d.hb_idx[6 * k + 4]) - (Rl)d.hb_nat[6 * k];
            if (fabs((double)rdev) > 2.0) {
                w.st[kl] = 1;
                for (int u = w.hb_off[kl]; u < w.hb_off[kl + 1]; ++u) atomicSub(w.exc + w.hb_pos[u], 1);
                w.en[kl] = 0.0;
            }
            int br;
            w.term[6 * kl] = (double)six_term<D>(P, d.hb_idx + 6 * k, d.hb_nat + 6 * k, 0, rdev, br);
        }
        // the angle and dihedral terms: warp task (chunk of 32 live bonds, term 1..5)
        const int nchunk = (nact + 31) >> 5;
        for (int task = warp; task < 5 * nchunk; task += nwarp) {
            const int s = 1 + task % 5, t = (task / 5) * 32 + lane;
            if (t < nact) {
                const int k = d.hb_active[hb0 + t], kl = k - hb0;
                int br;
                const Rl v = six_term<D>(P, d.hb_idx + 6 * k, d.hb_nat + 6 * k, s, Rl(0), br);
                w.term[6 * kl + s] = (double)v;
                if (s >= 3) w.br[3 * kl + s - 3] = br;
            }
        }
        bar();
        for (int t = tid; t < nact; t += bd) {
            const int k = d.hb_active[hb0 + t], kl = k - hb0;
            if (w.st[kl] == 1) continue;
            Rl q = Rl(0);
            for (int s = 0; s < 6; ++s) q += (Rl)w.term[6 * kl + s];
            w.en[kl] = (double)((Rl)d.hb_E[k] * exp_(-q));
            w.code[kl] = (w.br[3 * kl] + 1) + 3 * (w.br[3 * kl + 1] + 1) + 9 * (w.br[3 * kl + 2] + 1);
        }
        bar();
        lap(8);
        if (tid < 32) {  // valence-limited Monte Carlo (E:2239-2315), one warp
            const unsigned lt = (1u << lane) - 1u;
            unsigned long long ctr = s_ctr, vbase = ctr;
            fill_draws(s_v, R->seed, vbase, lane);
            const double T = R->T;
            const float inv_t = 1.0f / R->Tf;
            int guard = nact + 2;
            while (guard-- > 0) {
                // A: atoms with positive excess, in atom order
                int nA = 0;
                for (int base = 0; base < nca; base += 32) {
                    const int i = base + lane;
                    const bool pos = i < nca && w.exc[i] > 0;
                    const unsigned m = __ballot_sync(kFull, pos);
                    if (pos) w.al[nA + __popc(m & lt)] = i;
                    nA += __popc(m);
                }
                if (nA == 0) break;
                // draws ctr, ctr+1, ...: the atom, the K shuffle, the acceptances; u[i] is draw ctr + i
                if (ctr - vbase > 32) {
                    vbase = ctr;
                    fill_draws(s_v, R->seed, vbase, lane);
                }
                const uint32_t *u = s_v + (ctr - vbase);
                const int nu = 64 - (int)(ctr - vbase);  // draws held from u[0] on (at least 32)
                const int atom = w.al[pick_index(u[0], nA) - 1];
                // K: the atom's candidates still formed, in candidate order
                const int c0 = w.ca_off[atom], nc = w.ca_off[atom + 1] - c0;
                int nK = 0;
                for (int base = 0; base < nc; base += 32) {
                    const int t = base + lane;
                    const int k = t < nc ? w.ca_idx[c0 + t] : 0;
                    const bool ok = t < nc && w.st[k] == 0;
                    const unsigned m = __ballot_sync(kFull, ok);
                    if (ok) w.kl[nK + __popc(m & lt)] = k;
                    nK += __popc(m);
                }
                __syncwarp();
                if (nK == 0) {
                    ctr += 1;
                    A.err |= kErrRange;
                    break;
                }
                if (lane == 0)
                    for (int i = 1; i <= nK; ++i) {
                        const int jj = pick_index(i < nu ? u[i] : rand_value(R->seed, ctr + i), nK);
                        const int tmp = w.kl[i - 1];
                        w.kl[i - 1] = w.kl[jj - 1];
                        w.kl[jj - 1] = tmp;
                    }
                __syncwarp();
                // Metropolis walk over the shuffled K (draws nK+1 .. 2nK-1): lane a*nK+b
                // decides whether candidate a replaces candidate b
                int kc = 0;
                if (nK * nK <= 32) {
                    const int a = lane / nK, b = lane - a * nK;
                    const bool acc = lane < nK * nK && a >= 1 &&
                                     accept_move(u[nK + a], w.en[w.kl[a]], w.en[w.kl[b]], T, inv_t);
                    const unsigned dm = __ballot_sync(kFull, acc);
                    for (int a2 = 1; a2 < nK; ++a2)
                        if ((dm >> (a2 * nK + kc)) & 1u) kc = a2;
                } else if (lane == 0) {
                    for (int i = 2; i <= nK; ++i) {
                        const int di = nK + i - 1;
                        const uint32_t v = di < nu ? u[di] : rand_value(R->seed, ctr + di);
                        if (accept_move(v, w.en[w.kl[i - 1]], w.en[w.kl[kc]], T, inv_t)) kc = i - 1;
                    }
                }
                if (lane == 0) {
                    const int k = w.kl[kc];
                    w.st[k] = 1;
                    for (int u = w.hb_off[k]; u < w.hb_off[k + 1]; ++u) w.exc[w.hb_pos[u]] -= 1;
                }
                ctr += 2 * nK;
                __syncwarp();
            }
            if (lane == 0) s_ctr = ctr;
        }
        bar();
        lap(9);
        // forces of the bonds still formed: warp task (chunk of 32 live bonds, term 0..5)
        for (int task = warp; task < 6 * nchunk; task += nwarp) {
            const int s = task % 6, t = (task / 6) * 32 + lane;
            if (t < nact) {
                const int k = d.hb_active[hb0 + t], kl = k - hb0;
                if (w.st[kl] != 1) {
                    const Rl wk = -(Rl)w.en[kl];
                    if (s == 0) {
                        if (d.hb_dode[k]) e3hb -= (double)wk;
                        else e2hb -= (double)wk;
                    }
                    six_force_term<D>(P, A, d.hb_idx + 6 * k, d.hb_nat + 6 * k, w.code[kl], wk, s);
                }
            }
        }
    }
    if (do_hb && d.hb_rec)  // the bonds formed after the Monte Carlo (status 0; 1 broken, -1 out of range)
        for (int i = tid; i < nhb; i += bd) d.hb_rec[hb0 + i] = w.st[i] == 0 ? 1 : 0;
    lap(10);
    // ---- full_forces: the step's Gaussians follow the Monte Carlo draws ----
    const unsigned long long c1 = s_ctr;
    if (make_noise) gen_noise<D>(d, r, c1, tid, bd);
    if (d.fprof) {  // the Gaussians of every thread are done (timer runs only)
        bar();
        lap(11);
    }

    double v[2] = {e2hb, e3hb};
    block_sum_t<2>(v, s_red, tid, bd, bar);
    if (do_hb)
        for (int t = tid; t < nact; t += bd) {  // every live bond is formed again for the next step
            const int kl = d.hb_active[hb0 + t] - hb0;
            if (w.st[kl] == 1) w.st[kl] = 0;
        }
    if (tid == 0) {
        S->ctr = make_noise ? c1 + kNoise : c1;
        if (do_hb) { S->e2hb = v[0]; S->e3hb = v[1]; }
        if (EN) {
            double *e = d.eterm + r * kNE;
            e[8] += v[0]; e[9] += v[1];
        }
    }
    if (A.err) atomicOr(&S->err, A.err);
}

template <bool D, bool EN>
__global__ void __launch_bounds__(kHbThreads) k_hbond(Dev d, int do_hb, int make_noise)
{
    hbond_block<D, EN>(d, blockIdx.x, do_hb, make_noise, (int)threadIdx.x, (int)blockDim.x, CtaBar{});
}

__device__ void control_step(const Dev &d, int r);

// x < 0 and x > L (L > 0) on the bit patterns, as IEEE comparisons decide them for
// finite x (-0.0 is not below zero): integer instructions instead of FP64 compares
__device__ inline bool below_zero(double x)
{
    const long long b = __double_as_longlong(x);
    return b < 0 && b != (long long)0x8000000000000000ull;
}
__device__ inline bool above(double x, double L) { return __double_as_longlong(x) > __double_as_longlong(L); }

// |x| < 2^20 and finite, from the exponent field
__device__ inline bool bounded(double x)
{
    return ((unsigned)(__double_as_longlong(x) >> 52) & 0x7ffu) < 1023u + 20u;
}

// the recentring shift of adjust_box (E:2632-2656): the centre bead's new position
// moved to the box centre; one warp per replica, after every force is final
template <bool D>
__global__ void k_shift(Dev d)
{
    wait_prior_grid();
    const int r = blockIdx.x;
    const RepParams *R = d.rp + r;
    if (threadIdx.x == 0) {
        double xn[3], vn[3];
        leap_frog<D>(d, R, r, R->center, xn, vn);
        for (int c = 0; c < 3; ++c) d.shift[3 * r + c] = R->hbox[c] - xn[c];
    }
}

// The five Energies-file values of replica r (E:6308-6312: E2_HB, E3_HB, E2_STACK,
// E3_STACK of the last step, Rg of the RNA at the current positions) into out[0..4],
// by threads tid = 0 .. nthr-1 (written by tid 0)
template <class Bar>
__device__ void energies_block(const Dev &d, int r, double *out, int tid, int nthr, Bar bar)
{
    const RepParams *R = d.rp + r;
    __shared__ double s_red[3 * 32];
    __shared__ double s_c[3];
    double c[3] = {0, 0, 0};
    for (int i = tid; i < R->nrna; i += nthr) {
        c[0] += d.x[R->p0 + i];
        c[1] += d.y[R->p0 + i];
        c[2] += d.z[R->p0 + i];
    }
    block_sum_t<3>(c, s_red, tid, nthr, bar);
    if (tid == 0)
        for (int k = 0; k < 3; ++k) s_c[k] = c[k] / R->nrna;
    bar();
    double sq[1] = {0};
    for (int i = tid; i < R->nrna; i += nthr) {
        const double a = d.x[R->p0 + i] - s_c[0], b = d.y[R->p0 + i] - s_c[1], e = d.z[R->p0 + i] - s_c[2];
        sq[0] += a * a + b * b + e * e;
    }
    block_sum_t<1>(sq, s_red, tid, nthr, bar);
    if (tid == 0) {
        const RepState *S = d.rs + r;
        out[0] = S->e2hb;
        out[1] = S->e3hb;
        out[2] = S->e2st;
        out[3] = S->e3st;
        out[4] = sqrt(sq[0] / R->nrna);
    }
}

// The frame of replica r after step klok into its slot of the frame ring (d.fr),
// by threads tid = 0 .. nthr-1 of one block: positions, then the five energies,
// then, after a system-scope fence, the step number that marks the slot complete.
template <class Bar>
__device__ void write_frame(const Dev &d, int r, long long klok, int tid, int nthr, Bar bar)
{
    const FrameRing &F = d.fr;
    const RepParams *R = d.rp + r;
    const long long slot = (klok / F.every) % F.depth;
    const long long base = F.pk_base + R->pk0;
    double *px = F.pos + slot * 3 * F.n_total;
    for (int i = tid; i < R->n; i += nthr) {
        px[base + i] = d.x[R->p0 + i];
        px[F.n_total + base + i] = d.y[R->p0 + i];
        px[2 * F.n_total + base + i] = d.z[R->p0 + i];
    }
    __shared__ double s_e5[5];
    energies_block(d, r, s_e5, tid, nthr, bar);
    bar();
    if (tid < 5) F.en[(slot * F.R_total + F.rep_base + r) * 5 + tid] = s_e5[tid];
    __threadfence_system();
    bar();
    if (tid == 0) {
        __threadfence_system();
        *(volatile long long *)(F.done + slot * F.R_total + F.rep_base + r) = klok;
    }
}

// move_rigid_units for particle p of replica r (leap-frog, the recentring shift
// sh, the ions' periodic wrap, the new fixed-point position, its force sum zeroed);
// bits: max |x - x_old|^2 as bit pattern, err: flags
template <bool D>
__device__ __forceinline__ void integrate_particle(const Dev &d, const RepParams *R, int r, int p, const double sh[3],
                                                   unsigned long long &bits, int &err)
{
    const int4 qp = d.q[p];
    if (!((qp.w >> 16) & 1)) return;
    double xn[3], vn[3];
    leap_frog<D>(d, R, r, p, xn, vn);
    double xo[3] = {d.x[p], d.y[p], d.z[p]};
    for (int c = 0; c < 3; ++c) {
        xn[c] = xn[c] + sh[c];
        xo[c] = xo[c] + sh[c];
    }
    if (p - R->p0 >= R->nrna) {  // periodic wrap of the ions (E:2676-2731)
        for (int c = 0; c < 3; ++c) {
            if (below_zero(xn[c])) { xn[c] += R->box[c]; xo[c] += R->box[c]; }
            if (above(xn[c], R->box[c])) { xn[c] -= R->box[c]; xo[c] -= R->box[c]; }
        }
    }
    double e2 = 0.0;
    for (int c = 0; c < 3; ++c) {
        const double e = xn[c] - xo[c];
        e2 += e * e;
    }
    bits = max(bits, (unsigned long long)__double_as_longlong(e2));
    // a runaway or non-finite particle (|x| or |v| component >= 2^20) stops the run
    bool ok = true;
    for (int c = 0; c < 3; ++c) ok = ok && bounded(xn[c]) && bounded(vn[c]);
    if (!ok) err |= kErrNonFinite;
    d.x[p] = xn[0]; d.y[p] = xn[1]; d.z[p] = xn[2];
    d.xo[p] = xo[0]; d.yo[p] = xo[1]; d.zo[p] = xo[2];
    d.vx[p] = vn[0]; d.vy[p] = vn[1]; d.vz[p] = vn[2];
    d.f[p] = 0ull;  // consumed: the next step's force kernels accumulate from zero
    d.f[d.P + p] = 0ull;
    d.f[2 * d.P + p] = 0ull;
    int4 q = qp;  // floor(x L / 2^32) modulo 2^32, one rounding conversion per axis
    q.x = (int)(unsigned)__double2ll_rd(xn[0] * R->qinv[0]);
    q.y = (int)(unsigned)__double2ll_rd(xn[1] * R->qinv[1]);
    q.z = (int)(unsigned)__double2ll_rd(xn[2] * R->qinv[2]);
    d.q[p] = q;
}

// move_rigid_units (E:2660-2731) of one particle per thread: leap-frog, the
// recentring shift, the periodic wrap of the ions; the replica's last block to
// finish runs the skin check
// kIntPer particles per thread, kBlock / kIntPer threads per block of kBlock particles
template <bool D>
__global__ void __launch_bounds__(kBlock / kIntPer) k_integrate(Dev d)
{
    wait_prior_grid();
    const int r = d.blk_rep[blockIdx.x];
    const RepParams *R = d.rp + r;
    __shared__ unsigned long long s_max;
    if (threadIdx.x == 0) s_max = 0ull;
    __syncthreads();
    const double sh[3] = {d.shift[3 * r], d.shift[3 * r + 1], d.shift[3 * r + 2]};
    unsigned long long bits = 0ull;  // max |x - x_old|^2 of the thread's particles (non-negative doubles order as integers)
    int err = 0;
#pragma unroll
    for (int j = 0; j < kIntPer; ++j)
        integrate_particle<D>(d, R, r, blockIdx.x * kBlock + j * (kBlock / kIntPer) + threadIdx.x, sh, bits, err);
    // check_shifts (E:1745-1762): max |x - x_old|^2 over the block
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long b = __shfl_down_sync(kFull, bits, o);
        bits = b > bits ? b : bits;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(&s_max, bits);
    __syncthreads();
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        atomicMax(&d.rs[r].maxd2, s_max);
        __threadfence();
        // the replica's last block to finish runs the skin check for it
        const unsigned done = atomicAdd(&d.rs[r].blocks_done, 1u);
        s_last = (done == (unsigned)(R->npad / kBlock) - 1u);
        if (s_last) d.rs[r].blocks_done = 0u;
    }
    if (err) atomicOr(&d.rs[r].err, err);
    __syncthreads();
    if (s_last) {
        __threadfence();
        control_step(d, r);
        if (d.fr.every > 0) {  // a frame step: this block writes the replica's frame (all its blocks are done)
            __syncthreads();
            const long long kl = *(volatile long long *)&d.rs[r].klok;
            if (kl % d.fr.every == 0) write_frame(d, r, kl, (int)threadIdx.x, (int)blockDim.x, CtaBar{});
        }
    }
}

// check_shifts (E:1741-1776) and the LR gate of deterministic_forces_MPI (E:2550)
// for replica r, by thread 0.  RepState::rebuild stays as decided here until the
// next step's decision: the rebuild kernels that follow read it.
__device__ void control_step(const Dev &d, int r)
{
    const RepParams *R = d.rp + r;
    RepState *S = d.rs + r;
    if (threadIdx.x == 0) {
        const double d2 = __longlong_as_double((long long)atomicExch(&S->maxd2, 0ull));
        const double sh = sqrt(d2);
        S->progress += (sh + sh);
        S->klok += 1;
        int reb = S->progress > R->skin;
        if (reb) S->progress = 0.0;
        S->rebuild = reb;
        const long long kn = S->klok + 1;
        S->lr_now = (R->lr_interval <= 1) || (kn % R->lr_interval == 1) || (S->progress == 0.0);
        S->e2st = S->e2st_acc;  // stacking energies of the step just finished (E2_STACK, E3_STACK)
        S->e3st = S->e3st_acc;
        S->e2st_acc = 0.0;
        S->e3st_acc = 0.0;
    }
}

__global__ void k_force_rebuild(Dev d)
{
    RepState *S = d.rs + blockIdx.x;
    if (threadIdx.x == 0) {
        S->rebuild = 1;
        S->progress = 0.0;
        S->lr_now = 1;
        S->maxd2 = 0ull;
    }
}

// ---------------------------------------------------------------------------
// list rebuild (populate_lists, E:1546-1737)
// ---------------------------------------------------------------------------
// separate_in_cells (E:1461-1542): single periodic wrap then ceil(tmp / l)
__device__ inline int cell_axis(double v, double side, double l)
{
    double t = v;
    if (t < 0) t = __dadd_rn(t, side);
    else if (t > side) t = __dsub_rn(t, side);
    return (int)ceil(__ddiv_rn(t, l));
}

// cell_axis decided in FP32 from the fixed-point coordinate q = floor(v 2^32 / side)
// mod 2^32, for v in [0, side] (no wrap): c = q m / 2^32 approximates v / l (l = side
// / m) within 2e-7 m; when c lies farther than 4e-7 m + 1e-6 from an integer, ceil(c)
// is the FP64 result, else the FP64 form decides.
__device__ inline int cell_axis_q(double v, unsigned q, double side, double l, int m)
{
    const long long b = __double_as_longlong(v);
    if (b >= 0 && b <= __double_as_longlong(side)) {
        const float c = (float)q * ((float)m * 2.3283064365386963e-10f);
        const float fr = c - floorf(c), band = 4.0e-7f * (float)m + 1.0e-6f;
        if (fr > band && fr < 1.0f - band) return (int)c + 1;
    }
    return cell_axis(v, side, l);
}

// Work items of the replicas that rebuild this step, laid end to end (`per`: 0 =
// padded particles, 1 = cells).  Warp-collective: maps item i to its replica r and
// the offset within it; returns false past the end.
__device__ inline bool rebuild_item(const Dev &d, int per, int i, int &r, int &off)
{
    const int lane = threadIdx.x & 31;
    int acc = 0;
    for (int base = 0; base < d.R; base += 32) {
        const int rr = base + lane;
        const int n = (rr < d.R && d.rs[rr].rebuild) ? (per ? d.rp[rr].nc : d.rp[rr].npad) : 0;
        int incl = n;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += t;
        }
        const int tot = __shfl_sync(kFull, incl, 31);
        if (i < acc + tot) {
            const unsigned m = __ballot_sync(kFull, i < acc + incl);
            const int src = __ffs(m) - 1;
            r = base + src;
            off = i - acc - __shfl_sync(kFull, incl - n, src);
            return true;
        }
        acc += tot;
    }
    return false;
}

// populate_lists' cell binning (separate_in_cells, E:1461-1542) and hydrogen-bond
// candidate status (E:1698-1736) of one rebuilding replica per block.  Counting
// and filling run on shared-memory cell counters when the replica's cells fit
// (Dev::cell_smem), else on the global ones.  In FP64 mode each cell's particles
// are put in index order, as the reference appends them (E:1536-1540), so that
// list order and FP64 summation order are reproducible; mixed-precision sums are
// exact in fixed point and need no order.  Then the packed positions are copied
// in cell order, so the pair search reads each cell's candidates contiguously.
constexpr int kCellThreads = 1024;

template <bool D>
__device__ __forceinline__ void cells_block(const Dev &d, int r)
{
    extern __shared__ int s_cells[];
    __shared__ int s_warp[32];
    __shared__ int s_carry;
    RepState *S = d.rs + r;
    if (!S->rebuild) return;
    const RepParams *R = d.rp + r;
    const int nc = R->nc, tid = threadIdx.x, bd = blockDim.x, lane = tid & 31, w = tid >> 5, nw = bd >> 5;
    // per cell: particle count, first slot (in place of the count in shared memory), fill counter
    int *cnt = d.cell_smem ? s_cells : d.cell_count + R->c0;
    int *first = d.cell_smem ? s_cells : d.cell_start + R->c0;
    int *fill = d.cell_smem ? s_cells + d.nc_max : d.cell_fill + R->c0;
    for (int c = tid; c < nc; c += bd) {
        cnt[c] = 0;
        fill[c] = 0;
    }
    if (tid == 0) s_carry = 0;
    __syncthreads();
    for (int i = tid; i < R->npad; i += bd) {
        const int p = R->p0 + i;
        int c = -1;
        const int4 qp = d.q[p];
        if ((qp.w >> 16) & 1) {
            const int i1 = cell_axis_q(d.x[p], (unsigned)qp.x, R->box[0], R->lcell[0], R->mc[0]);
            const int i2 = cell_axis_q(d.y[p], (unsigned)qp.y, R->box[1], R->lcell[1], R->mc[1]);
            const int i3 = cell_axis_q(d.z[p], (unsigned)qp.z, R->box[2], R->lcell[2], R->mc[2]);
            if (i1 < 1 || i1 > R->mc[0] || i2 < 1 || i2 > R->mc[1] || i3 < 1 || i3 > R->mc[2]) {
                atomicOr(&S->err, kErrRange);
            } else {
                c = (i1 - 1) * R->mc[1] * R->mc[2] + (i2 - 1) * R->mc[2] + (i3 - 1);
                atomicAdd(cnt + c, 1);
            }
        }
        d.cell_of[p] = c;
    }
    __syncthreads();
    // exclusive scan of the counts: first slot of every cell
    for (int base = 0; base < nc; base += bd) {
        const int c = base + tid;
        const int v = c < nc ? cnt[c] : 0;
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_warp[w] = incl;
        __syncthreads();
        if (w == 0) {
            int t = lane < nw ? s_warp[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(kFull, t, o);
                if (lane >= o) t += u;
            }
            if (lane < nw) s_warp[lane] = t;
        }
        __syncthreads();
        const int excl = s_carry + (w > 0 ? s_warp[w - 1] : 0) + incl - v;
        if (c < nc) {
            first[c] = excl;
            d.cell_start[R->c0 + c] = excl;
            d.cell_count[R->c0 + c] = v;
        }
        __syncthreads();
        if (tid == bd - 1) s_carry = excl + v;
        __syncthreads();
    }
    const int nslots = s_carry;
    for (int i = tid; i < R->npad; i += bd) {
        const int p = R->p0 + i;
        const int c = d.cell_of[p];
        if (c >= 0) d.cell_list[R->p0 + first[c] + atomicAdd(fill + c, 1)] = p;
    }
    __syncthreads();
    if (D)  // one warp per cell: rank sort (at most 8 particles per lane), or insertion sort by one lane
        for (int c = w; c < nc; c += nw) {
            const int n = d.cell_count[R->c0 + c];
            int *seg = d.cell_list + R->p0 + first[c];
            if (n > 1 && n <= 256) {
                int v[8], rk[8];
                int m = 0;
                for (int i = lane; i < n; i += 32, ++m) {
                    v[m] = seg[i];
                    int k = 0;
                    for (int u = 0; u < n; ++u) k += seg[u] < v[m];
                    rk[m] = k;
                }
                __syncwarp();
                for (int t = 0; t < m; ++t) seg[rk[t]] = v[t];
                __syncwarp();
            } else if (n > 256) {
                if (lane == 0)
                    for (int i = 1; i < n; ++i) {
                        const int v = seg[i];
                        int j = i - 1;
                        while (j >= 0 && seg[j] > v) {
                            seg[j + 1] = seg[j];
                            --j;
                        }
                        seg[j + 1] = v;
                    }
                __syncwarp();
            }
        }
    __syncthreads();
    for (int i = tid; i < nslots; i += bd) d.qs[R->p0 + i] = d.q[d.cell_list[R->p0 + i]];

    // hydrogen-bond candidates: live (0) when the central pair is within the SR radius
    for (int a = R->hba0 + tid; a < R->hba1; a += bd) d.hb_excess[a] = d.hba_n[a] - d.hba_val[a];
    __syncthreads();
    for (int k = R->hb0 + tid; k < R->hb1; k += bd) {
        const int a = d.hb_idx[6 * k + 1], b = d.hb_idx[6 * k + 4];
        const int st = (a != b && exact_r2(d, R, a, b) <= R->r2sr) ? 0 : -1;
        d.hb_status[k] = st;
        if (st != 0)
            for (int u = d.hb_aoff[k]; u < d.hb_aoff[k + 1]; ++u) atomicSub(d.hb_excess + d.hb_aidx[u], 1);
    }
    if (tid == 0) s_carry = 0;
    __syncthreads();
    // ordered compaction of the live candidates
    const int nh = R->hb1 - R->hb0;
    for (int base = 0; base < nh; base += bd) {
        const int k = R->hb0 + base + tid;
        const bool live = (base + tid < nh) && d.hb_status[k] == 0;
        const unsigned m = __ballot_sync(kFull, live);
        if (lane == 0) s_warp[w] = __popc(m);
        __syncthreads();
        int off = s_carry;
        for (int t = 0; t < w; ++t) off += s_warp[t];
        if (live) d.hb_active[R->hb0 + off + __popc(m & ((1u << lane) - 1u))] = k;
        __syncthreads();
        if (tid == 0) {
            int tot = 0;
            for (int t = 0; t < nw; ++t) tot += s_warp[t];
            s_carry += tot;
        }
        __syncthreads();
    }
    if (tid == 0) {
        S->n_active = s_carry;
        S->rebuilds += 1;
    }
}

template <bool D>
__global__ void __launch_bounds__(kCellThreads) k_cells(Dev d)
{
    wait_prior_grid();
    cells_block<D>(d, blockIdx.x);
}

// distinct periodic neighbours of cell index i (1..m) along one axis
__device__ inline int axis_neighbours(int i, int m, int out[3])
{
    int n = 0;
    for (int dd = -1; dd <= 1; ++dd) {
        int v = i + dd;
        if (v < 1) v += m;
        if (v > m) v -= m;
        bool dup = false;
        for (int t = 0; t < n; ++t) dup |= (out[t] == v);
        if (!dup) out[n++] = v;
    }
    return n;
}

// SR and LR neighbour lists (E:1576-1694).  A pair is SR when r^2 <= (sr+skin)^2,
// else LR when r^2 <= (rc+skin)^2 and neither bead is a sugar or a base.  The FP32
// distance from the exact integer differences decides outside a narrow band
// around each threshold; inside it the FP64 distance with the reference's
// rounding and image rule decides, so the lists are the reference's sets.
// One warp per particle: the lanes scan a neighbour cell's candidates together
// (contiguous in cell order) and append hits in candidate order by ballot.  The
// warps stride over the particles of the replicas that rebuild this step.
// populate_lists' pair search for particle `off` of replica r by one warp; pre, beg:
// the warp's 32 + 32 ints of shared memory
template <bool D>
__device__ __forceinline__ void search_particle(const Dev &d, int r, int off, int lane, int *pre, int *beg)
{
    const unsigned lt = (1u << lane) - 1u;
    const int P = d.P;
    const RepParams *R = d.rp + r;
    const float sx = R->qstep[0], sy = R->qstep[1], sz = R->qstep[2];
    const float sr_lo = R->r2srf * (1.0f - kBand), sr_hi = R->r2srf * (1.0f + kBand);
    const float lr_lo = R->r2lrf * (1.0f - kBand), lr_hi = R->r2lrf * (1.0f + kBand);
    {
        const int p = R->p0 + off;
        const int c = d.cell_of[p];
        if (c < 0) {
            if (lane == 0) { d.n_sr[p] = 0; d.n_lr[p] = 0; }
            return;
        }
        const int4 qp = d.q[p];
        const bool chp = is_charged((qp.w >> 8) & 0xff);
        const int i1 = c / (R->mc[1] * R->mc[2]) + 1, i2 = (c / R->mc[2]) % R->mc[1] + 1, i3 = c % R->mc[2] + 1;
        int n1[3], n2[3], n3[3];
        const int m1 = axis_neighbours(i1, R->mc[0], n1);
        const int m2 = axis_neighbours(i2, R->mc[1], n2);
        const int m3 = axis_neighbours(i3, R->mc[2], n3);
        int exl[kExcl];
        const int nex = d.n_excl[p];
        for (int t2 = 0; t2 < kExcl; ++t2) exl[t2] = t2 < nex ? d.excl[(size_t)t2 * P + p] : -1;
        // the neighbour cells' candidate ranges laid end to end, in the reference's
        // cell order (lane s < 27 holds cell s of the 3 x 3 x 3 block)
        const int nseg = m1 * m2 * m3;
        __syncwarp();  // the previous particle's reads of pre/beg are done
        int cnt_l = 0, start_l = 0;
        if (lane < nseg) {
            const int a = lane / (m2 * m3), b = (lane / m3) % m2, e = lane % m3;
            const int cc = (n1[a] - 1) * R->mc[1] * R->mc[2] + (n2[b] - 1) * R->mc[2] + (n3[e] - 1);
            start_l = R->p0 + d.cell_start[R->c0 + cc];
            cnt_l = d.cell_count[R->c0 + cc];
        }
        int incl = cnt_l;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        if (lane < nseg) {
            pre[lane] = incl - cnt_l;
            beg[lane] = start_l;
        }
        if (lane == 0) pre[nseg] = total;
        __syncwarp();
        int nsr = 0, nlr = 0, seg = 0;
        constexpr int kU = 4;  // candidate chunks of 32 whose loads are issued together
        for (int t0 = 0; t0 < total; t0 += 32 * kU) {
            int jv[kU];
            int4 qv[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int t = t0 + 32 * u + lane;
                jv[u] = -1;
                qv[u] = make_int4(0, 0, 0, 0);
                if (t < total) {
                    while (t >= pre[seg + 1]) ++seg;
                    const int slot = beg[seg] + (t - pre[seg]);
                    jv[u] = d.cell_list[slot];
                    qv[u] = d.qs[slot];
                }
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                if (t0 + 32 * u >= total) break;
                const int j = jv[u];
                const int4 qj = qv[u];
                int cls = 0;  // 0 none, 1 SR, 2 LR
                if (j >= 0 && j != p) {
                    const bool ch = chp && is_charged((qj.w >> 8) & 0xff);
                    const float dx = (float)(int)((unsigned)qp.x - (unsigned)qj.x) * sx;
                    const float dy = (float)(int)((unsigned)qp.y - (unsigned)qj.y) * sy;
                    const float dz = (float)(int)((unsigned)qp.z - (unsigned)qj.z) * sz;
                    const float r2f = dx * dx + dy * dy + dz * dz;
                    if (D) {
                        const double r2 = exact_r2(d, R, p, j);
                        cls = r2 <= R->r2sr ? 1 : ((ch && r2 <= R->r2lr) ? 2 : 0);
                    } else {
                        if (r2f < sr_lo) cls = 1;
                        else if (r2f > sr_hi && (!ch || r2f > lr_hi)) cls = 0;
                        else if (r2f > sr_hi && r2f < lr_lo) cls = 2;
                        else {
                            const double e2 = exact_r2(d, R, p, j);
                            cls = e2 <= R->r2sr ? 1 : ((ch && e2 <= R->r2lr) ? 2 : 0);
                        }
                    }
                    // pruned list: a pair with an uncharged bead can only exert LJ, which
                    // vanishes beyond D_LJ; the skin keeps it exact until the next rebuild
                    if (cls == 1 && !d.full_lists && !ch && r2f > R->ljkeep2[jn12(qp.w & 0xff, qj.w & 0xff)])
                        cls = 0;
                }
                const unsigned bs = __ballot_sync(kFull, cls == 1), bl = __ballot_sync(kFull, cls == 2);
                if (cls == 1) {
                    int m = 0;  // how often the reference subtracts this pair's LJ again
                    for (int t2 = 0; t2 < nex; ++t2) m += (exl[t2] == j);
                    const int pos = nsr + __popc(bs & lt);
                    if (pos < d.cap_sr) d.nbr_sr[nb_idx(pos, p, P)] = j | (m << kExclShift);
                } else if (cls == 2) {
                    const int pos = nlr + __popc(bl & lt);
                    if (pos < d.cap_lr) d.nbr_lr[nb_idx(pos, p, P)] = j;
                }
                nsr += __popc(bs);
                nlr += __popc(bl);
            }
        }
        if (lane == 0) {
            if (nsr > d.cap_sr || nlr > d.cap_lr) atomicOr(&d.rs[r].err, kErrCapacity);
            d.n_sr[p] = min(nsr, d.cap_sr);
            d.n_lr[p] = min(nlr, d.cap_lr);
        }
    }
}

template <bool D>
__global__ void __launch_bounds__(128) k_pair_search(Dev d)
{
    wait_prior_grid();
    __shared__ int s_pre[4][32], s_beg[4][32];  // per warp: candidate offsets and first slots of its cells
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int r, off;
    for (int item = wid; rebuild_item(d, 0, item, r, off); item += d.search_warps)
        search_particle<D>(d, r, off, lane, s_pre[threadIdx.x >> 5], s_beg[threadIdx.x >> 5]);
}

// ---------------------------------------------------------------------------
// persistent fused step kernel: one thread-block cluster per replica runs `steps`
// whole steps (the sequence of E:6380-6386) without leaving the kernel
// ---------------------------------------------------------------------------
// A replica's cluster of C CTAs (cluster dimension C, grid R x C) shares its work;
// phases are separated by the cluster's hardware barrier (all CTAs of a cluster are
// resident together, so no wait depends on another cluster).  Per step:
//   forces   warps 0-7 of the first CTA: H-bond terms, the valence-limited Monte
//            Carlo and the step's Gaussians (hbond_block on a named barrier); all
//            other threads: SR pairs (one thread per particle), LR pairs when due
//            (four per particle), bonded terms and stacks (one thread per item)
//   shift    every CTA forms the recentring shift from the centre bead
//   move     each CTA integrates its share of the particles; max |x - x_old|^2
//   control  check_shifts and the LR gate (control_step) by the first CTA
//   rebuild  when due: cell binning by the first CTA, pair search by every warp
// Data the kernel rewrites while it runs is read through L2 (ld_in<true>, __ldcg).
constexpr int kFusedThreads = 512;
constexpr int kFusedHbThreads = 256;
constexpr int kFusedWarps = kFusedThreads / 32;

__device__ __forceinline__ int cluster_rank()
{
    unsigned v;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(v));
    return (int)v;
}
__device__ __forceinline__ int cluster_ctas()
{
    unsigned v;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(v));
    return (int)v;
}
// every thread of the cluster; writes before it (global and shared) are visible to
// every thread of the cluster after it
__device__ __forceinline__ void cluster_barrier()
{
    __threadfence();
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

template <bool D>
__global__ void __launch_bounds__(kFusedThreads, 1) k_step_fused(Dev d, int steps)
{
    const int cs = cluster_ctas(), rank = cluster_rank();
    const int r = blockIdx.x / cs;
    const RepParams *R = d.rp + r;
    RepState *S = d.rs + r;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ float s_dlj2[46], s_dm[46], s_flj[46], s_qclb[46];
    __shared__ int s_pre[kFusedWarps][32], s_beg[kFusedWarps][32];
    __shared__ double s_shift[3];
    __shared__ unsigned long long s_max;
    for (int t = tid; t < 46; t += kFusedThreads) {
        s_dlj2[t] = R->dlj2[t];
        s_dm[t] = R->dm[t];
        s_flj[t] = R->flj[t];
        s_qclb[t] = R->qclb[t];
    }
    __syncthreads();
    const PairTables tb{s_dlj2, s_dm, s_flj, s_qclb};
    const bool hbt = rank == 0 && tid < kFusedHbThreads;  // the H-bond threads
    const int nwk = cs * kFusedThreads - kFusedHbThreads;  // pair workers (a multiple of 32)
    const int wk = rank * kFusedThreads + tid - kFusedHbThreads;  // this thread's worker index (when !hbt)
    const int npad = R->npad, p0 = R->p0;
    const int nb = R->bt1 - R->bt0, n3 = R->s31 - R->s30, n2 = R->s21 - R->s20;
    const int per = (npad / kBlock + cs - 1) / cs * kBlock;  // particles integrated per CTA
    int err = 0;
    // phase times (tis_profile_fused): the first thread of the cluster's first CTA
    const bool timer = d.fprof && rank == 0 && tid == 0;
    unsigned long long ph[8] = {0, 0, 0, 0, 0, 0, 0, 0}, t0 = timer ? global_ns() : 0ull, t1;
    auto lap = [&](int k) {
        if (timer) {
            t1 = global_ns();
            ph[k] += t1 - t0;
            t0 = t1;
        }
    };
    for (int step = 0; step < steps; ++step) {
        const int lr_now = __ldcg(&S->lr_now);
        if (hbt) {
            hbond_block<D, false>(d, r, 1, 1, tid, kFusedHbThreads, NamedBar{1, kFusedHbThreads});
            if (timer) ph[1] += global_ns() - t0;
        } else {
            double e0 = 0, e1 = 0;
            for (int i = wk; i < npad; i += nwk) pair_particle<D, false, false, true, 1, true>(d, R, p0 + i, 0, tb, err, e0, e1);
            if (lr_now)  // groups of four workers per particle (every group of a warp runs the same passes)
                for (int i = wk >> 2; i < npad; i += nwk >> 2)
                    pair_particle<D, true, false, false, 4, true>(d, R, p0 + i, wk & 3, tb, err, e0, e1);
            for (int i = wk; i < nb + n3 + n2; i += nwk) {
                const int t = i < nb ? R->bt0 + i
                                     : (i < nb + n3 ? d.nbt + R->s30 + (i - nb) : d.nbt + d.nst3 + R->s20 + (i - nb - n3));
                topo_item<D, false>(d, t, 4 | 8, 1);
            }
        }
        cluster_barrier();
        lap(0);
        ph[6] += lr_now ? 1 : 0;
        if (tid == 0) {  // adjust_box's shift (E:2632-2656) from the centre bead's new position
            double xn[3], vn[3];
            leap_frog<D>(d, R, r, R->center, xn, vn);
            for (int c = 0; c < 3; ++c) s_shift[c] = R->hbox[c] - xn[c];
            if (rank == 0)
                for (int c = 0; c < 3; ++c) d.shift[3 * r + c] = s_shift[c];  // as k_shift leaves it
            s_max = 0ull;
        }
        cluster_barrier();  // no CTA moves the centre bead before every CTA has read it
        lap(2);
        {
            const double sh[3] = {s_shift[0], s_shift[1], s_shift[2]};
            unsigned long long bits = 0ull;
            const int i1 = min(npad, (rank + 1) * per);
            for (int i = rank * per + tid; i < i1; i += kFusedThreads) integrate_particle<D>(d, R, r, p0 + i, sh, bits, err);
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long b = __shfl_down_sync(kFull, bits, o);
                bits = b > bits ? b : bits;
            }
            if (lane == 0) atomicMax(&s_max, bits);
            __syncthreads();
            if (tid == 0) atomicMax(&S->maxd2, s_max);
        }
        cluster_barrier();
        lap(3);
        if (rank == 0) control_step(d, r);  // thread 0: check_shifts, the next step's LR gate
        cluster_barrier();
        lap(4);
        if (d.fr.every > 0 && rank == 0) {  // a frame step: the first CTA writes the replica's frame
            const long long kl = __ldcg(&S->klok);
            if (kl % d.fr.every == 0) write_frame(d, r, kl, tid, kFusedThreads, CtaBar{});
        }
        if (__ldcg(&S->rebuild)) {  // populate_lists (E:1546-1737)
            if (rank == 0) cells_block<D>(d, r);
            cluster_barrier();
            for (int off = rank * kFusedWarps + warp; off < npad; off += cs * kFusedWarps)
                search_particle<D>(d, r, off, lane, s_pre[warp], s_beg[warp]);
            cluster_barrier();
            lap(5);
            ph[7] += 1;
        }
    }
    if (err) atomicOr(&S->err, err);
    if (timer)
        for (int k = 0; k < 8; ++k) atomicAdd(d.fprof + (size_t)r * kFusedPhases + k, ph[k]);
}

// radius_of_gyration (E:2844-2876) of the RNA beads of one replica
__global__ void k_rg(Dev d, int r, double *out)
{
    const RepParams *R = d.rp + r;
    __shared__ double s_red[3 * 32];
    double c[3] = {0, 0, 0};
    for (int i = threadIdx.x; i < R->nrna; i += blockDim.x) {
        c[0] += d.x[R->p0 + i];
        c[1] += d.y[R->p0 + i];
        c[2] += d.z[R->p0 + i];
    }
    block_sum<3>(c, s_red);
    __shared__ double s_c[3];
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) s_c[k] = c[k] / R->nrna;
    __syncthreads();
    double s[1] = {0};
    for (int i = threadIdx.x; i < R->nrna; i += blockDim.x) {
        const double a = d.x[R->p0 + i] - s_c[0], b = d.y[R->p0 + i] - s_c[1], e = d.z[R->p0 + i] - s_c[2];
        s[0] += a * a + b * b + e * e;
    }
    block_sum<1>(s, s_red);
    if (threadIdx.x == 0) *out = sqrt(s[0] / R->nrna);
}

// Ions of one kind within sqrt(r2cut) of each phosphate of replica r, from the SR
// lists (complete within the SR radius between rebuilds): count[i] for RNA bead i
// (-1 for sugars and bases), hit[j] = 1 for every ion j within range of some P.
__global__ void k_ion_counts(Dev d, int r, int kind, double r2cut, int *count, int *hit)
{
    const RepParams *R = d.rp + r;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R->nrna) return;
    const int p = R->p0 + i;
    if (((d.q[p].w >> 8) & 0xff) != 0) {
        count[i] = -1;
        return;
    }
    int c = 0;
    for (int k = 0; k < d.n_sr[p]; ++k) {
        const int j = d.nbr_sr[nb_idx(k, p, d.P)] & kIdxMask;
        if (((d.q[j].w >> 8) & 0xff) == kind && exact_r2(d, R, p, j) <= r2cut) {
            ++c;
            hit[j - R->p0] = 1;
        }
    }
    count[i] = c;
}

// clears every replica's device-side error flags
__global__ void k_clear_err(Dev d)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < d.R; r += gridDim.x * blockDim.x) d.rs[r].err = 0;
}

// the largest SR and LR neighbour counts of the group (out[0], out[1]; zero on entry)
__global__ void k_list_peaks(Dev d, int *out)
{
    int a = 0, b = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < d.P; p += gridDim.x * blockDim.x) {
        a = max(a, d.n_sr[p]);
        b = max(b, d.n_lr[p]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        a = max(a, __shfl_down_sync(kFull, a, o));
        b = max(b, __shfl_down_sync(kFull, b, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, a);
        atomicMax(out + 1, b);
    }
}

// E2_HB, E3_HB, E2_STACK, E3_STACK and Rg of every replica (one block each)
__global__ void k_energies(Dev d, double *out)
{
    energies_block(d, blockIdx.x, out + 5 * blockIdx.x, (int)threadIdx.x, (int)blockDim.x, CtaBar{});
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_quantize(const Dev &d, cudaStream_t s) { k_quantize<<<d.nblk, kBlock, 0, s>>>(d); }

void launch_put_state(const Dev &d, cudaStream_t s, const double *stage, int n)
{
    k_put_state<<<d.nblk, kBlock, 0, s>>>(d, stage, n);
}

void launch_get_state(const Dev &d, cudaStream_t s, double *stage, int n, unsigned mask)
{
    k_get_state<<<d.nblk, kBlock, 0, s>>>(d, stage, n, mask);
}

void launch_energies(const Dev &d, cudaStream_t s, double *out) { k_energies<<<d.R, 256, 0, s>>>(d, out); }

void launch_clear_err(const Dev &d, cudaStream_t s) { k_clear_err<<<1, 256, 0, s>>>(d); }

void launch_list_peaks(const Dev &d, cudaStream_t s, int *out) { k_list_peaks<<<d.sm_count, 256, 0, s>>>(d, out); }

void launch_ion_counts(const Dev &d, cudaStream_t s, int r, int nrna, int kind, double r2cut, int *count, int *hit)
{
    k_ion_counts<<<(nrna + 127) / 128, 128, 0, s>>>(d, r, kind, r2cut, count, hit);
}

void launch_pair_sr(const Dev &d, cudaStream_t s, bool en, bool ex)
{
    constexpr int L = kLanesSR, T = kBlock * kLanesSR;
    if (!en && ex && d.lanes_sr == 2) {  // the step's SR launch in the other shapes (tis_run_params.lanes_sr)
        if (d.fp64) k_pair<true, false, false, true, 2, 2 * kBlock><<<d.nblk, 2 * kBlock, 0, s>>>(d, 1);
        else k_pair<false, false, false, true, 2, 2 * kBlock><<<d.nblk, 2 * kBlock, 0, s>>>(d, 1);
        return;
    }
    if (!en && ex && d.lanes_sr == 4) {
        if (d.fp64) k_pair<true, false, false, true, 4, 4 * kBlock><<<d.nblk, 4 * kBlock, 0, s>>>(d, 1);
        else k_pair<false, false, false, true, 4, 4 * kBlock><<<d.nblk, 4 * kBlock, 0, s>>>(d, 1);
        return;
    }
    if (d.fp64) {
        if (en) k_pair<true, false, true, false, L, T><<<d.nblk, T, 0, s>>>(d, 1);
        else if (ex) k_pair<true, false, false, true, L, T><<<d.nblk, T, 0, s>>>(d, 1);
        else k_pair<true, false, false, false, L, T><<<d.nblk, T, 0, s>>>(d, 1);
    } else {
        if (en) k_pair<false, false, true, false, L, T><<<d.nblk, T, 0, s>>>(d, 1);
        else if (ex) k_pair<false, false, false, true, L, T><<<d.nblk, T, 0, s>>>(d, 1);
        else k_pair<false, false, false, false, L, T><<<d.nblk, T, 0, s>>>(d, 1);
    }
}

void launch_pair_lr(const Dev &d, cudaStream_t s, bool en, bool force_all)
{
    constexpr int L = kLanesLR, T = kThreadsLR;
    const int fa = force_all ? 1 : 0;
    if (!en && d.lanes_lr == 2) {  // the step's LR launch in the other shapes (tis_run_params.lanes_lr)
        if (d.fp64) k_pair<true, true, false, false, 2, 2 * kBlock><<<d.nblk, 2 * kBlock, 0, s>>>(d, fa);
        else k_pair<false, true, false, false, 2, 2 * kBlock><<<d.nblk, 2 * kBlock, 0, s>>>(d, fa);
        return;
    }
    if (!en && d.lanes_lr == 8) {
        if (d.fp64) k_pair<true, true, false, false, 8, 8 * kBlock><<<d.nblk, 8 * kBlock, 0, s>>>(d, fa);
        else k_pair<false, true, false, false, 8, 8 * kBlock><<<d.nblk, 8 * kBlock, 0, s>>>(d, fa);
        return;
    }
    if (d.fp64) {
        if (en) k_pair<true, true, true, false, L, T><<<d.nblk, T, 0, s>>>(d, fa);
        else k_pair<true, true, false, false, L, T><<<d.nblk, T, 0, s>>>(d, fa);
    } else {
        if (en) k_pair<false, true, true, false, L, T><<<d.nblk, T, 0, s>>>(d, fa);
        else k_pair<false, true, false, false, L, T><<<d.nblk, T, 0, s>>>(d, fa);
    }
}

void launch_topology(const Dev &d, cudaStream_t s, int mask, bool en, bool make_noise, bool ex)
{
    const int xl = ex ? 1 : 0;
    const int items = d.nbt + d.nst3 + d.nst2;
    const int blocks = (items + kTopoThreads - 1) / kTopoThreads;
    if ((mask & (4 | 8)) && blocks > 0) {
        if (d.fp64) {
            if (en) k_bonded_stack<true, true><<<blocks, kTopoThreads, 0, s>>>(d, mask, xl);
            else k_bonded_stack<true, false><<<blocks, kTopoThreads, 0, s>>>(d, mask, xl);
        } else {
            if (en) k_bonded_stack<false, true><<<blocks, kTopoThreads, 0, s>>>(d, mask, xl);
            else k_bonded_stack<false, false><<<blocks, kTopoThreads, 0, s>>>(d, mask, xl);
        }
    }
    const int hb = (mask & 16) ? 1 : 0, mn = make_noise ? 1 : 0;
    const size_t sm = hb ? (size_t)d.hb_smem : 0;
    if (hb || mn) {
        if (d.fp64) {
            if (en) k_hbond<true, true><<<d.R, kHbThreads, sm, s>>>(d, hb, mn);
            else k_hbond<true, false><<<d.R, kHbThreads, sm, s>>>(d, hb, mn);
        } else {
            if (en) k_hbond<false, true><<<d.R, kHbThreads, sm, s>>>(d, hb, mn);
            else k_hbond<false, false><<<d.R, kHbThreads, sm, s>>>(d, hb, mn);
        }
    }
}

int configure_kernels(const Dev &d)
{
    cudaError_t e = cudaSuccess;
    if (fused_smem(d) > 48 * 1024) {
        const int b = (int)fused_smem(d);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_step_fused<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_step_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    }
    if (d.cell_smem > 48 * 1024) {
        const int b = d.cell_smem;
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cells<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cells<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    }
    if (d.hb_smem > 48 * 1024) {
        const int b = d.hb_smem;
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_hbond<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_hbond<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_hbond<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_hbond<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    }
    return (int)e;
}

void launch_noise(const Dev &d, cudaStream_t s)
{
    if (d.fp64) k_noise<true><<<d.R, kTopoThreads, 0, s>>>(d);
    else k_noise<false><<<d.R, kTopoThreads, 0, s>>>(d);
}

// a launch that may begin before the previous kernel on the stream has finished
// (the kernel waits in wait_prior_grid)
template <class K>
void launch_pdl(K kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t s, const Dev &d)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, d);
}

void launch_shift(const Dev &d, cudaStream_t s)
{
    if (d.fp64) launch_pdl(k_shift<true>, d.R, 32, 0, s, d);
    else launch_pdl(k_shift<false>, d.R, 32, 0, s, d);
}

void launch_move(const Dev &d, cudaStream_t s)
{
    if (d.fp64) launch_pdl(k_integrate<true>, d.nblk, kBlock / kIntPer, 0, s, d);
    else launch_pdl(k_integrate<false>, d.nblk, kBlock / kIntPer, 0, s, d);
}

void launch_integrate(const Dev &d, cudaStream_t s)
{
    launch_shift(d, s);
    launch_move(d, s);
}

void launch_cells(const Dev &d, cudaStream_t s)
{
    if (d.fp64) launch_pdl(k_cells<true>, d.R, kCellThreads, d.cell_smem, s, d);
    else launch_pdl(k_cells<false>, d.R, kCellThreads, d.cell_smem, s, d);
}

void launch_search(const Dev &d, cudaStream_t s)
{
    if (d.fp64) launch_pdl(k_pair_search<true>, d.search_warps / 4, 128, 0, s, d);
    else launch_pdl(k_pair_search<false>, d.search_warps / 4, 128, 0, s, d);
}

void launch_rebuild(const Dev &d, cudaStream_t s)
{
    launch_cells(d, s);
    launch_search(d, s);
}

void launch_force_all_rebuild(const Dev &d, cudaStream_t s) { k_force_rebuild<<<d.R, 128, 0, s>>>(d); }

void launch_rg(const Dev &d, cudaStream_t s, int replica, double *out) { k_rg<<<1, 256, 0, s>>>(d, replica, out); }

// pair SR, pair LR, bonded+stacking, H-bonds (+Gaussians), shift, integrate (+skin check), cells, pair search
int kernel_launches_per_step() { return 8; }

size_t fused_smem(const Dev &d) { return (size_t)max(d.hb_smem, d.cell_smem); }

int launch_step_fused(const Dev &d, cudaStream_t s, int steps, int ctas)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(d.R * ctas));
    cfg.blockDim = dim3(kFusedThreads);
    cfg.dynamicSmemBytes = fused_smem(d);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return (int)(d.fp64 ? cudaLaunchKernelEx(&cfg, k_step_fused<true>, d, steps)
                        : cudaLaunchKernelEx(&cfg, k_step_fused<false>, d, steps));
}

}  // namespace tis
