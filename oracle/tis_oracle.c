/* TEST INFRASTRUCTURE — FP64 CPU oracle of the TIS-RNA Langevin step.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it.
 *
 * Every function restates one routine of the reference engine
 * (E: = src/16SCD_Mg_Cl_K_COPY_fast.cpp of naotohori/16S-central-folding) and
 * cites the lines it follows.  Arithmetic is written in the reference's
 * evaluation order where that order decides rounding (pair distances, list
 * thresholds, pair forces), so pair sets are bit-identical and forces agree to
 * rounding.  The hydrogen-bond Monte Carlo and the noise consume the shared
 * Philox rand() stream (oracle_rng.h) in the reference's call order.
 * Build with -ffp-contract=off. */
#include "tis_oracle.h"
#include "oracle_rng.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NA 9
#define NPA 45
static const double PI = 3.14159265358979323846264338328;
static const double SIG0 = 1.5852; /* LJ length scale used throughout E:749-821 */

typedef struct { int32_t *v; int64_t n, cap; } ivec;

static void ivec_push2(ivec *a, int32_t p, int32_t q)
{
    if (a->n + 2 > a->cap) {
        a->cap = a->cap ? 2 * a->cap : 4096;
        a->v = (int32_t *)realloc(a->v, (size_t)a->cap * sizeof(int32_t));
    }
    a->v[a->n++] = p;
    a->v[a->n++] = q;
}

struct tis_o {
    tis_o_desc d;
    /* owned copies of the topology */
    int32_t *type, *kind;
    int32_t *bt_kind, *bt_a, *bt_b, *bt_c; double *bt_k0, *bt_x0;
    int32_t *st3_idx, *st3_off; double *st3_native, *st3_E;
    int32_t *st2_idx; double *st2_r0, *st2_E;
    int32_t *hb_idx, *hb_dode, *hb_atom_off, *hb_atom_idx; double *hb_native, *hb_E;
    int32_t *hba_valence, *hba_cand_off, *hba_cand_idx;
    /* parameter tables (E:2883-2945), index 1..9 / 1..45 as in the reference */
    double MASS[NA + 1], VISC[NA + 1], K1[NA + 1], K2[NA + 1], SIGMA[NA + 1];
    double D_LJ[NPA + 1], D2_CUT[NPA + 1], D2_MIN[NPA + 1], E_LJ[NPA + 1], F_LJ[NPA + 1], Q_C[NPA + 1];
    double hX, hY, hZ, D2_CT, R2_SR, R2_LR;
    /* state */
    double *x, *y, *z, *xo, *yo, *zo, *vx, *vy, *vz;
    double *fx, *fy, *fz, *flx, *fly, *flz;
    /* lists */
    int32_t McX, McY, McZ;
    int32_t *cell_of, *cell_start, *cell_list;
    ivec sr, lr;
    /* hydrogen bonds */
    int32_t *hb_status, *HB_EXCESS, *EXCESS, *HB_ATOM_N, *hb_A, *hb_K;
    double *hb_energy, *hb_psi0;  /* 3 per candidate */
    int64_t *pair_key; int32_t *pair_cand; /* candidates sorted by central-pair key */
    /* stacks */
    double *st_energy; int32_t *st_status;
    /* run */
    int64_t klok, rebuilds;
    double PROGRESS;
    uint64_t ctr;
    double E2_HB, E3_HB, E2_STACK, E3_STACK;
};

static void *dupm(const void *p, size_t n)
{
    void *q = malloc(n ? n : 1);
    if (n) memcpy(q, p, n);
    return q;
}

static int jn12(int a, int b) /* E:1803-1805 */
{
    if (a < b) return (a - 1) * NA - (a - 1) * a / 2 + b;
    return (b - 1) * NA - (b - 1) * b / 2 + a;
}

static int o_rand(tis_o *o) { return tis_o_rand_value(o->d.seed, 0u, o->ctr++); }

/* ---- geometry (E:646-670, E:986-1027, E:1255-1302) ------------------------ */
static void half_shift(const tis_o *o, double *v) /* E:646-653 */
{
    if (v[0] > o->hX) v[0] = v[0] - o->d.box[0];
    if (v[0] < -o->hX) v[0] = v[0] + o->d.box[0];
    if (v[1] > o->hY) v[1] = v[1] - o->d.box[1];
    if (v[1] < -o->hY) v[1] = v[1] + o->d.box[1];
    if (v[2] > o->hZ) v[2] = v[2] - o->d.box[2];
    if (v[2] < -o->hZ) v[2] = v[2] + o->d.box[2];
}

static double image_r2(const tis_o *o, int i, int j, double *v) /* CC_vector + r^2 (E:674-683) */
{
    v[0] = o->x[i] - o->x[j];
    v[1] = o->y[i] - o->y[j];
    v[2] = o->z[i] - o->z[j];
    half_shift(o, v);
    return v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
}

static double distance(const tis_o *o, int i, int j) /* CC_distance, no image (E:657-670) */
{
    double a = o->x[i] - o->x[j], b = o->y[i] - o->y[j], c = o->z[i] - o->z[j];
    return sqrt(a * a + b * b + c * c);
}

static double angle_of(const tis_o *o, int i1, int i2, int i3) /* valence_angle (E:986-1027) */
{
    double a[3] = { o->x[i1] - o->x[i2], o->y[i1] - o->y[i2], o->z[i1] - o->z[i2] };
    double b[3] = { o->x[i3] - o->x[i2], o->y[i3] - o->y[i2], o->z[i3] - o->z[i2] };
    double na = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    double nb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
    double c = (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) / sqrt(na * nb);
    return acos(c);
}

static void cross(const double *a, const double *b, double *r)
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

static double dot(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static void bond_vec(const tis_o *o, int from, int to, double *v)
{
    v[0] = o->x[to] - o->x[from];
    v[1] = o->y[to] - o->y[from];
    v[2] = o->z[to] - o->z[from];
}

static double dihedral_of(const tis_o *o, int i1, int i2, int i3, int i4) /* dihedral_angle (E:1255-1302) */
{
    double v1[3], v2[3], v3[3], m[3], n[3];
    bond_vec(o, i1, i2, v1);
    bond_vec(o, i2, i3, v2);
    bond_vec(o, i3, i4, v3);
    cross(v1, v2, m);
    cross(v2, v3, n);
    double l2 = sqrt(dot(v2, v2));
    return atan2(dot(v1, n) * l2, dot(m, n));
}

/* ---- pair forces and energies (E:749-855) --------------------------------- */
static double lj_force(const tis_o *o, double r2, int J) /* LJ_FORCE (E:801-821) */
{
    if (r2 > o->D2_CUT[J]) return 0;
    double r1 = sqrt(r2);
    double dr = r1 + SIG0 - o->D_LJ[J];
    double s = SIG0 / dr;
    double s2 = s * s, s4 = s2 * s2, s8 = s4 * s4, s14 = s8 * s4 * s2;
    return o->F_LJ[J] * (s14 - s8) * dr / r1;
}

/* COULOMB_TRUNCATED_FORCE (E:841-855); with a Debye length lambda (no counterpart in
 * the reference) the screened form U = Q lB exp(-r / lambda) / r, whose force over
 * r is U (1 + r / lambda) / r^2 */
static double coulomb_force(const tis_o *o, double r2, int J)
{
    if (r2 > o->D2_CT) return 0;
    double r1 = sqrt(r2);
    if (o->d.debye > 0.0 && isfinite(o->d.debye)) {
        double kr = r1 / o->d.debye, u = o->Q_C[J] * o->d.lB * exp(-kr) / r1;
        return u * (1.0 + kr) / r2;
    }
    return o->Q_C[J] * o->d.lB / (r1 * r2);
}

static double wca_energy(const tis_o *o, double r2, int J) /* WCA_ENERGY (E:749-771) */
{
    if (r2 > o->D2_CUT[J]) return 0;
    if (r2 < o->D2_MIN[J]) return o->E_LJ[J] * 1001.0;
    double r1 = sqrt(r2);
    double dr = r1 + SIG0 - o->D_LJ[J];
    double s = SIG0 / dr;
    double s2 = s * s, s4 = s2 * s2, s6 = s4 * s2, s12 = s6 * s6;
    return o->E_LJ[J] * (s12 - 2.0 * s6 + 1.0);
}

static double coulomb_energy(const tis_o *o, double r2, int J) /* COULOMB_TRUNCATED_ENERGY (E:825-837) */
{
    if (r2 > o->D2_CT) return 0;
    if (o->d.debye > 0.0 && isfinite(o->d.debye)) {
        double r1 = sqrt(r2);
        return o->Q_C[J] * o->d.lB * exp(-r1 / o->d.debye) / r1;
    }
    return o->Q_C[J] * o->d.lB / sqrt(r2);
}

static int charged(const tis_o *o, int i) { return o->kind[i] != 1 && o->kind[i] != 2; }

/* exclusion: subtract the LJ force of a bonded pair (reduce_forces, E:880-897) */
static void exclude_lj(tis_o *o, int i, int j)
{
    double v[3];
    double r2 = image_r2(o, i, j, v);
    double s = -1.0 * lj_force(o, r2, jn12(o->type[i], o->type[j]));
    v[0] *= s; v[1] *= s; v[2] *= s;
    o->fx[i] += v[0]; o->fx[j] -= v[0];
    o->fy[i] += v[1]; o->fy[j] -= v[1];
    o->fz[i] += v[2]; o->fz[j] -= v[2];
}

/* harmonic bond k0 (r0 - r)^2 (bead_bond_force / stacking_bond_force, E:924-982) */
static void bond_force(tis_o *o, int i1, int i2, double k0, double r0)
{
    double v[3];
    bond_vec(o, i1, i2, v);
    double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double t = 2.0 * k0 * (r0 - r) / r;
    double a = t * v[0], b = t * v[1], c = t * v[2];
    o->fx[i1] -= a; o->fx[i2] += a;
    o->fy[i1] -= b; o->fy[i2] += b;
    o->fz[i1] -= c; o->fz[i2] += c;
}

/* harmonic angle k0 (theta0 - theta)^2 at i2 (bead_valence_force E:1031-1134,
 * stacking_valence_force E:1138-1251).  The force is s * d(cos theta)/dx with
 * s = -2 k0 (theta0 - theta) / sin theta.  clamp=1 applies the stacking
 * variant's guard: cos < -0.99995 gives theta = pi and no force. */
static void angle_force(tis_o *o, int i1, int i2, int i3, double k0, double th0, int clamp)
{
    double a[3] = { o->x[i1] - o->x[i2], o->y[i1] - o->y[i2], o->z[i1] - o->z[i2] };
    double b[3] = { o->x[i3] - o->x[i2], o->y[i3] - o->y[i2], o->z[i3] - o->z[i2] };
    double ia = 1.0 / (a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    double ib = 1.0 / (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    double iab = sqrt(ia * ib);
    double c = (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) * iab;
    double sn, th;
    if (clamp && c < -0.99995) { sn = 0; th = PI; }
    else { sn = sqrt(1.0 - c * c); th = acos(c); }
    double s = 0;
    if (!clamp || sn != 0) s = -2.0 * k0 * (th0 - th) / sn;
    double ca = c * ia, cb = c * ib;
    for (int k = 0; k < 3; ++k) {
        double g1 = b[k] * iab - a[k] * ca;          /* d cos / d x1 */
        double g3 = a[k] * iab - b[k] * cb;          /* d cos / d x3 */
        double g2 = -(a[k] + b[k]) * iab + a[k] * ca + b[k] * cb;
        double *f = k == 0 ? o->fx : (k == 1 ? o->fy : o->fz);
        f[i1] += s * g1;
        f[i2] += s * g2;
        f[i3] += s * g3;
    }
}

/* harmonic dihedral k0 (psi0 - psi)^2 (stacking_dihedral_force, E:1306-1454):
 * s * d(cos psi)/dx with s = -2 k0 (psi0 - psi) / sin psi, cos psi = m.n/(|m||n|),
 * m = v1 x v2, n = v2 x v3. */
static void dihedral_force(tis_o *o, int i1, int i2, int i3, int i4, double k0, double psi0)
{
    double v1[3], v2[3], v3[3], m[3], n[3];
    bond_vec(o, i1, i2, v1);
    bond_vec(o, i2, i3, v2);
    bond_vec(o, i3, i4, v3);
    cross(v1, v2, m);
    cross(v2, v3, n);
    double im = 1.0 / dot(m, m), in = 1.0 / dot(n, n);
    double imn = sqrt(im * in);
    double l2 = sqrt(dot(v2, v2));
    double c = dot(m, n) * imn;
    double sn = dot(v1, n) * l2 * imn;
    double psi = atan2(sn, c);
    double s = -2.0 * k0 * (psi0 - psi) / sn;
    double cm = c * im, cn = c * in;
    double v2n[3], nv1[3], v3m[3], mv2[3], v2m[3], mv1[3], v3n[3], nv2[3];
    cross(v2, n, v2n); cross(n, v1, nv1); cross(v3, m, v3m); cross(m, v2, mv2);
    cross(v2, m, v2m); cross(m, v1, mv1); cross(v3, n, v3n); cross(n, v2, nv2);
    for (int k = 0; k < 3; ++k) {
        double G1 = v2n[k] * imn - cm * v2m[k];
        double G2 = (nv1[k] + v3m[k]) * imn - cm * mv1[k] - cn * v3n[k];
        double G3 = mv2[k] * imn - cn * nv2[k];
        double *f = k == 0 ? o->fx : (k == 1 ? o->fy : o->fz);
        f[i1] += s * (-G1);
        f[i2] += s * (G1 - G2);
        f[i3] += s * (G2 - G3);
        f[i4] += s * G3;
    }
}

static double image_psi0(double psi, double nat) /* E:1999-2019 */
{
    if (fabs(psi - nat) <= PI) return nat;
    if (psi - nat > PI) return nat + 2.0 * PI;
    return nat - 2.0 * PI;
}

/* ---- lists (E:1461-1737) --------------------------------------------------- */
static int cell_axis(double v, double side, double l) /* single wrap + ceil (E:1502-1530) */
{
    double t = v;
    if (t < 0) t += side;
    else if (t > side) t -= side;
    return (int)ceil(t / l);
}

static int pair_key_cmp(const void *a, const void *b)
{
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return x < y ? -1 : (x > y);
}

int tis_o_populate_lists(tis_o *o)
{
    const double lr = o->d.rc + o->d.skin;
    o->McX = (int)(o->d.box[0] / lr);
    o->McY = (int)(o->d.box[1] / lr);
    o->McZ = (int)(o->d.box[2] / lr);
    const double lX = o->d.box[0] / o->McX, lY = o->d.box[1] / o->McY, lZ = o->d.box[2] / o->McZ;
    const int McT = o->McX * o->McY * o->McZ;
    free(o->cell_start);
    o->cell_start = (int32_t *)calloc((size_t)McT + 2, sizeof(int32_t));
    for (int i = 0; i < o->d.n; ++i) { /* separate_in_cells (E:1461-1542) */
        int i1 = cell_axis(o->x[i], o->d.box[0], lX);
        int i2 = cell_axis(o->y[i], o->d.box[1], lY);
        int i3 = cell_axis(o->z[i], o->d.box[2], lZ);
        int m = (i1 - 1) * o->McY * o->McZ + (i2 - 1) * o->McZ + i3; /* 1-based */
        if (m < 1 || m > McT) return 1; /* the reference indexes out of its cell table here */
        o->cell_of[i] = m - 1;
        o->cell_start[m] += 1;
    }
    for (int m = 1; m <= McT + 1; ++m) o->cell_start[m] += o->cell_start[m - 1];
    {
        int32_t *fill = (int32_t *)calloc((size_t)McT + 1, sizeof(int32_t));
        for (int i = 0; i < o->d.n; ++i) { /* particles enter their cell in index order */
            int c = o->cell_of[i];
            o->cell_list[o->cell_start[c] + fill[c]++] = i;
        }
        free(fill);
    }
    static const int off[13][3] = { { -1, -1, -1 }, { -1, -1, 0 }, { -1, -1, 1 }, { -1, 0, -1 }, { -1, 0, 0 },
                                    { -1, 0, 1 }, { -1, 1, -1 }, { -1, 1, 0 }, { -1, 1, 1 }, { 0, -1, -1 },
                                    { 0, -1, 0 }, { 0, -1, 1 }, { 0, 0, -1 } }; /* E:1560-1562 */
    o->sr.n = 0;
    o->lr.n = 0;
    double v[3];
    for (int m1 = 1; m1 <= o->McX; ++m1)
    for (int m2 = 1; m2 <= o->McY; ++m2)
    for (int m3 = 1; m3 <= o->McZ; ++m3) {
        int J1 = (m1 - 1) * o->McY * o->McZ + (m2 - 1) * o->McZ + m3 - 1;
        for (int k = 0; k < 14; ++k) {
            int J2;
            if (k < 13) { /* half shell with the reference's wrap-and-skip rule (E:1586-1604) */
                int n1 = m1 + off[k][0], n2 = m2 + off[k][1], n3 = m3 + off[k][2];
                if (n1 > o->McX) { n1 -= o->McX; if (n1 == m1 || n1 == m1 - 1) continue; }
                else if (n1 < 1) { n1 += o->McX; if (n1 == m1 || n1 == m1 + 1) continue; }
                if (n2 > o->McY) { n2 -= o->McY; if (n2 == m2 || n2 == m2 - 1) continue; }
                else if (n2 < 1) { n2 += o->McY; if (n2 == m2 || n2 == m2 + 1) continue; }
                if (n3 > o->McZ) { n3 -= o->McZ; if (n3 == m3 || n3 == m3 - 1) continue; }
                else if (n3 < 1) { n3 += o->McZ; if (n3 == m3 || n3 == m3 + 1) continue; }
                J2 = (n1 - 1) * o->McY * o->McZ + (n2 - 1) * o->McZ + n3 - 1;
            } else {
                J2 = J1; /* intra-cell pairs j2 > j1 (E:1662-1691) */
            }
            for (int a = o->cell_start[J1]; a < o->cell_start[J1 + 1]; ++a) {
                int i1 = o->cell_list[a];
                int b0 = (J2 == J1) ? a + 1 : o->cell_start[J2];
                for (int b = b0; b < o->cell_start[J2 + 1]; ++b) {
                    int i2 = o->cell_list[b];
                    double r2 = image_r2(o, i1, i2, v);
                    if (r2 <= o->R2_SR) ivec_push2(&o->sr, i1, i2);
                    else if (r2 <= o->R2_LR && charged(o, i1) && charged(o, i2)) ivec_push2(&o->lr, i1, i2);
                }
            }
        }
    }
    /* hydrogen-bond candidate status (E:1698-1725): -1 unless the candidate's
     * central pair is in the SR list; HB_PAIR is a sort of candidates by pair key. */
    for (int k = 0; k < o->d.n_hb; ++k) o->hb_status[k] = -1;
    const int64_t NR = o->d.n_rna;
    for (int64_t p = 0; p < o->sr.n; p += 2) {
        int i1 = o->sr.v[p], i2 = o->sr.v[p + 1];
        if (o->kind[i1] > 2 || o->kind[i2] > 2) continue;
        int64_t key = i1 < i2 ? (int64_t)i1 * NR + i2 : (int64_t)i2 * NR + i1;
        int lo = 0, hi = o->d.n_hb;
        while (lo < hi) { int md = (lo + hi) / 2; if (o->pair_key[md] < key) lo = md + 1; else hi = md; }
        for (int q = lo; q < o->d.n_hb && o->pair_key[q] == key; ++q) o->hb_status[o->pair_cand[q]] = 0;
    }
    for (int a = 0; a < o->d.n_hba; ++a) o->HB_EXCESS[a] = o->HB_ATOM_N[a] - o->d.hba_valence[a]; /* E:1729 */
    for (int k = 0; k < o->d.n_hb; ++k) {
        if (o->hb_status[k] == 0) continue;
        for (int t = o->hb_atom_off[k]; t < o->hb_atom_off[k + 1]; ++t) o->HB_EXCESS[o->hb_atom_idx[t]] -= 1;
    }
    o->rebuilds += 1;
    return 0;
}

/* ---- force terms ----------------------------------------------------------- */
static void sr_forces(tis_o *o, double *elj, double *ecoul) /* SR_interactions_lists (E:1783-1847) */
{
    double v[3];
    for (int64_t p = 0; p < o->sr.n; p += 2) {
        int i = o->sr.v[p], j = o->sr.v[p + 1];
        int J = jn12(o->type[i], o->type[j]);
        double r2 = image_r2(o, i, j, v);
        double t = lj_force(o, r2, J);
        int ch = charged(o, i) && charged(o, j);
        if (ch) t += coulomb_force(o, r2, J);
        if (elj) { *elj += wca_energy(o, r2, J); if (ch) *ecoul += coulomb_energy(o, r2, J); }
        v[0] *= t; v[1] *= t; v[2] *= t;
        o->fx[i] += v[0]; o->fx[j] -= v[0];
        o->fy[i] += v[1]; o->fy[j] -= v[1];
        o->fz[i] += v[2]; o->fz[j] -= v[2];
    }
}

static void lr_forces(tis_o *o, double *ecoul) /* LR_interactions_lists (E:1851-1907) */
{
    double v[3];
    for (int64_t p = 0; p < o->lr.n; p += 2) {
        int i = o->lr.v[p], j = o->lr.v[p + 1];
        int J = jn12(o->type[i], o->type[j]);
        double r2 = image_r2(o, i, j, v);
        double t = coulomb_force(o, r2, J);
        if (ecoul) *ecoul += coulomb_energy(o, r2, J);
        v[0] *= t; v[1] *= t; v[2] *= t;
        o->flx[i] += v[0]; o->flx[j] -= v[0];
        o->fly[i] += v[1]; o->fly[j] -= v[1];
        o->flz[i] += v[2]; o->flz[j] -= v[2];
    }
}

static void bonded_forces(tis_o *o, double *e) /* polymer_constraints (E:2354-2520) */
{
    double v[3];
    for (int t = 0; t < o->d.n_bt; ++t) {
        int a = o->bt_a[t], b = o->bt_b[t], c = o->bt_c[t];
        if (o->bt_kind[t] == 0) {
            bond_force(o, a, b, o->bt_k0[t], o->bt_x0[t]);
            exclude_lj(o, a, b);
            if (e) {
                double r = distance(o, a, b);
                e[0] += o->bt_k0[t] * (r - o->bt_x0[t]) * (r - o->bt_x0[t]);
                e[2] -= wca_energy(o, image_r2(o, a, b, v), jn12(o->type[a], o->type[b]));
            }
        } else {
            angle_force(o, a, b, c, o->bt_k0[t], o->bt_x0[t], 0);
            exclude_lj(o, a, c);
            if (e) {
                double th = angle_of(o, a, b, c);
                e[1] += o->bt_k0[t] * (th - o->bt_x0[t]) * (th - o->bt_x0[t]);
                e[2] -= wca_energy(o, image_r2(o, a, c, v), jn12(o->type[a], o->type[c]));
            }
        }
    }
}

/* six-term native-geometry restraint shared by tertiary stacks and hydrogen
 * bonds (E:2000-2056, E:2319-2349): bond 5w, angles 1.5w, dihedrals 0.15w */
static void six_term_forces(tis_o *o, const int32_t *k, const double *nat, const double *psi0s, double w)
{
    bond_force(o, k[1], k[4], 5.00 * w, nat[0]);
    angle_force(o, k[0], k[1], k[4], 1.50 * w, nat[1], 1);
    angle_force(o, k[3], k[4], k[1], 1.50 * w, nat[2], 1);
    dihedral_force(o, k[0], k[1], k[4], k[3], 0.15 * w, psi0s[0]);
    dihedral_force(o, k[4], k[1], k[0], k[2], 0.15 * w, psi0s[1]);
    dihedral_force(o, k[1], k[4], k[3], k[5], 0.15 * w, psi0s[2]);
}

/* geometry of the six-term restraint: returns the quadratic form Q and the imaged
 * native dihedrals (E:1983-2040, E:2177-2231) */
static double six_term_q(const tis_o *o, const int32_t *k, const double *nat, double r_dev, double *psi0s,
                         double init)
{
    double t1 = angle_of(o, k[0], k[1], k[4]);
    double t2 = angle_of(o, k[3], k[4], k[1]);
    double p = dihedral_of(o, k[0], k[1], k[4], k[3]);
    double p1 = dihedral_of(o, k[4], k[1], k[0], k[2]);
    double p2 = dihedral_of(o, k[1], k[4], k[3], k[5]);
    psi0s[0] = image_psi0(p, nat[3]);
    psi0s[1] = image_psi0(p1, nat[4]);
    psi0s[2] = image_psi0(p2, nat[5]);
    double q = init + 5.00 * r_dev * r_dev;
    q += 1.50 * (t1 - nat[1]) * (t1 - nat[1]);
    q += 1.50 * (t2 - nat[2]) * (t2 - nat[2]);
    q += 0.15 * (p - psi0s[0]) * (p - psi0s[0]);
    q += 0.15 * (p1 - psi0s[1]) * (p1 - psi0s[1]);
    q += 0.15 * (p2 - psi0s[2]) * (p2 - psi0s[2]);
    return q;
}

static void stacking(tis_o *o) /* stacking_interactions (E:1911-2141) */
{
    const int n3 = o->d.n_st3, n2 = o->d.n_st2;
    for (int k = 0; k < n3 + n2; ++k) { o->st_energy[k] = 0; o->st_status[k] = 0; }
    double psi0s[3];
    for (int k = 0; k < n3; ++k) {
        const int32_t *id = o->st3_idx + 6 * k;
        const double *nat = o->st3_native + 6 * k;
        double r = distance(o, id[1], id[4]) - nat[0];
        if (r < 10.0) { /* switch off the secondary stacks sharing a site (E:1960-1981) */
            for (int s = 0; s < 2; ++s) {
                int t = o->st3_off[2 * k + s];
                if (t >= 0) o->st_status[n3 + t] = 1;
            }
        }
        double D = six_term_q(o, id, nat, r, psi0s, 1.0);
        o->st_energy[k] = o->st3_E[k] / D;
        double w = -o->st_energy[k] / D;
        six_term_forces(o, id, nat, psi0s, w);
        o->E3_STACK += o->st_energy[k];
    }
    for (int k = 0; k < n2; ++k) {
        if (o->st_status[n3 + k]) continue;
        const int32_t *id = o->st2_idx + 7 * k; /* k_10 k00 k01 k10 k20 k21 k30 */
        double r = distance(o, id[2], id[5]);
        double p1 = dihedral_of(o, id[0], id[1], id[3], id[4]);
        double p2 = dihedral_of(o, id[6], id[4], id[3], id[1]);
        double p10 = image_psi0(p1, -2.58684), p20 = image_psi0(p2, 3.07135);
        double D = 1.0 + 1.40 * (r - o->st2_r0[k]) * (r - o->st2_r0[k]);
        D += 4.00 * (p1 - p10) * (p1 - p10);
        D += 4.00 * (p2 - p20) * (p2 - p20);
        double E = o->st2_E[k] / D;
        o->st_energy[n3 + k] = E;
        double w = -E / D;
        bond_force(o, id[2], id[5], 1.40 * w, o->st2_r0[k]);
        dihedral_force(o, id[0], id[1], id[3], id[4], 4.00 * w, p10);
        dihedral_force(o, id[6], id[4], id[3], id[1], 4.00 * w, p20);
        o->E2_STACK += E;
    }
}

static void hydrogen_bonds(tis_o *o) /* hydrogen_bonds_interactions (E:2145-2350) */
{
    const int nh = o->d.n_hb, na = o->d.n_hba;
    memcpy(o->EXCESS, o->HB_EXCESS, sizeof(int32_t) * (size_t)na);
    for (int k = 0; k < nh; ++k) o->hb_energy[k] = 0;
    for (int k = 0; k < nh; ++k) {
        if (o->hb_status[k] == -1) continue;
        const int32_t *id = o->hb_idx + 6 * k;
        const double *nat = o->hb_native + 6 * k;
        double r = distance(o, id[1], id[4]);
        if (fabs(r - nat[0]) > 2.0) {
            o->hb_status[k] = 1;
            for (int t = o->hb_atom_off[k]; t < o->hb_atom_off[k + 1]; ++t) o->EXCESS[o->hb_atom_idx[t]] -= 1;
            continue;
        }
        double q = six_term_q(o, id, nat, r - nat[0], o->hb_psi0 + 3 * k, 0.0);
        o->hb_energy[k] = o->hb_E[k] * exp(-q);
    }
    /* valence-limited Monte Carlo (E:2239-2315) */
    for (;;) {
        int nA = 0;
        for (int a = 0; a < na; ++a) if (o->EXCESS[a] > 0) o->hb_A[++nA] = a;
        if (nA == 0) break;
        double r = (double)o_rand(o) / TIS_O_RAND_MAX;
        int j = (int)ceil(r * nA);
        if (j == nA + 1) j = nA;
        if (j == 0) j = 1;
        int atom = o->hb_A[j];
        int nK = 0;
        for (int t = o->hba_cand_off[atom]; t < o->hba_cand_off[atom + 1]; ++t) {
            int k = o->hba_cand_idx[t];
            if (o->hb_status[k] == 0) o->hb_K[++nK] = k;
        }
        for (int i = 1; i <= nK; ++i) { /* shuffle */
            r = (double)o_rand(o) / TIS_O_RAND_MAX;
            j = (int)ceil(r * nK);
            if (j == nK + 1) j = nK;
            if (j == 0) j = 1;
            int tmp = o->hb_K[i]; o->hb_K[i] = o->hb_K[j]; o->hb_K[j] = tmp;
        }
        int k = o->hb_K[1];
        for (int i = 2; i <= nK; ++i) {
            int c = o->hb_K[i];
            double acc = exp((o->hb_energy[c] - o->hb_energy[k]) / o->d.T);
            r = (double)o_rand(o) / TIS_O_RAND_MAX;
            if (r < acc) k = c;
        }
        o->hb_status[k] = 1;
        for (int t = o->hb_atom_off[k]; t < o->hb_atom_off[k + 1]; ++t) o->EXCESS[o->hb_atom_idx[t]] -= 1;
    }
    for (int k = 0; k < nh; ++k) {
        if (o->hb_status[k] == -1) continue;
        if (o->hb_status[k] == 1) { o->hb_status[k] = 0; continue; }
        double w = -o->hb_energy[k];
        if (o->hb_dode[k]) o->E3_HB -= w; else o->E2_HB -= w;
        six_term_forces(o, o->hb_idx + 6 * k, o->hb_native + 6 * k, o->hb_psi0 + 3 * k, w);
    }
}

static double radius_of_gyration(const tis_o *o) /* E:2844-2876 over the RNA beads */
{
    double cx = 0, cy = 0, cz = 0, r = 0;
    int N = o->d.n_rna;
    for (int i = 0; i < N; ++i) { cx += o->x[i]; cy += o->y[i]; cz += o->z[i]; }
    cx /= N; cy /= N; cz /= N;
    for (int i = 0; i < N; ++i) {
        double a = o->x[i] - cx, b = o->y[i] - cy, c = o->z[i] - cz;
        r += a * a + b * b + c * c;
    }
    return sqrt(r / N);
}

/* ---- step ------------------------------------------------------------------ */
static void zero3(double *a, double *b, double *c, int n)
{
    memset(a, 0, sizeof(double) * (size_t)n);
    memset(b, 0, sizeof(double) * (size_t)n);
    memset(c, 0, sizeof(double) * (size_t)n);
}

static void deterministic_forces(tis_o *o) /* E:2524-2586 (one rank: the Allreduce is a copy) */
{
    int n = o->d.n;
    zero3(o->fx, o->fy, o->fz, n);
    o->E2_HB = o->E3_HB = o->E2_STACK = o->E3_STACK = 0;
    stacking(o);
    hydrogen_bonds(o);
    bonded_forces(o, NULL);
    sr_forces(o, NULL, NULL);
    if ((o->klok % o->d.lr_interval) == 1 || o->PROGRESS == 0) {
        zero3(o->flx, o->fly, o->flz, n);
        lr_forces(o, NULL);
    }
    for (int i = 0; i < n; ++i) { o->fx[i] += o->flx[i]; o->fy[i] += o->fly[i]; o->fz[i] += o->flz[i]; }
}

static void full_forces(tis_o *o) /* Langevin noise (E:2590-2625) */
{
    double g[3001];
    for (int i = 1; i < 3001; i += 2) {
        double r1 = (double)o_rand(o) / TIS_O_RAND_MAX; /* never 0 with this stream */
        double r2 = (double)o_rand(o) / TIS_O_RAND_MAX;
        double a = sqrt(-2.0 * log(r1)), b = 2.0 * PI * r2;
        g[i] = a * cos(b);
        g[i + 1] = a * sin(b);
    }
    if (!o->d.noise) return;
    for (int p = 0; p < o->d.n; ++p) {
        int t = o->type[p], k = (p + 1) % 1000; /* reference particle i = p + 1 */
        o->fx[p] = o->fx[p] + g[k + 1] * o->SIGMA[t];
        o->fy[p] = o->fy[p] + g[k + 1001] * o->SIGMA[t];
        o->fz[p] = o->fz[p] + g[k + 2001] * o->SIGMA[t];
    }
}

static void move(tis_o *o) /* move_rigid_units (E:2660-2732) with leap_frog_move_atom (E:570-642) */
{
    const double h = o->d.h, T = o->d.T;
    for (int k = 0; k < o->d.n; ++k) {
        int l = o->type[k];
        double x0 = o->x[k], y0 = o->y[k], z0 = o->z[k];
        double u = o->vx[k], v = o->vy[k], w = o->vz[k];
        o->vx[k] = o->K1[l] * u + o->K2[l] * o->fx[k];
        o->vy[k] = o->K1[l] * v + o->K2[l] * o->fy[k];
        o->vz[k] = o->K1[l] * w + o->K2[l] * o->fz[k];
        double vsq = o->MASS[l] * (o->vx[k] * o->vx[k] + o->vy[k] * o->vy[k] + o->vz[k] * o->vz[k]) / (300.0 * T);
        if (vsq > 1.0) {
            vsq = 1.0 / sqrt(vsq);
            o->vx[k] *= vsq; o->vy[k] *= vsq; o->vz[k] *= vsq;
        }
        o->x[k] = 2.0 * x0 - o->xo[k] + (o->vx[k] - u) * h;
        o->y[k] = 2.0 * y0 - o->yo[k] + (o->vy[k] - v) * h;
        o->z[k] = 2.0 * z0 - o->zo[k] + (o->vz[k] - w) * h;
        o->xo[k] = x0; o->yo[k] = y0; o->zo[k] = z0;
    }
    int c = o->d.center; /* adjust_box (E:2632-2656) */
    double dx = o->hX - o->x[c], dy = o->hY - o->y[c], dz = o->hZ - o->z[c];
    for (int k = 0; k < o->d.n; ++k) {
        o->x[k] += dx; o->xo[k] += dx;
        o->y[k] += dy; o->yo[k] += dy;
        o->z[k] += dz; o->zo[k] += dz;
    }
    for (int k = o->d.n_rna; k < o->d.n; ++k) { /* periodic wrap of the ions (E:2676-2731) */
        if (o->x[k] < 0) { o->x[k] += o->d.box[0]; o->xo[k] += o->d.box[0]; }
        if (o->x[k] > o->d.box[0]) { o->x[k] -= o->d.box[0]; o->xo[k] -= o->d.box[0]; }
        if (o->y[k] < 0) { o->y[k] += o->d.box[1]; o->yo[k] += o->d.box[1]; }
        if (o->y[k] > o->d.box[1]) { o->y[k] -= o->d.box[1]; o->yo[k] -= o->d.box[1]; }
        if (o->z[k] < 0) { o->z[k] += o->d.box[2]; o->zo[k] += o->d.box[2]; }
        if (o->z[k] > o->d.box[2]) { o->z[k] -= o->d.box[2]; o->zo[k] -= o->d.box[2]; }
    }
}

static void check_shifts(tis_o *o) /* E:1741-1776 */
{
    double shift = 0;
    for (int i = 0; i < o->d.n; ++i) {
        double a = o->x[i] - o->xo[i], b = o->y[i] - o->yo[i], c = o->z[i] - o->zo[i];
        double r2 = a * a + b * b + c * c;
        if (r2 > shift) shift = r2;
    }
    shift = sqrt(shift);
    o->PROGRESS += (shift + shift);
    if (o->PROGRESS > o->d.skin) {
        tis_o_populate_lists(o);
        o->PROGRESS = 0;
    }
}

void tis_o_step(tis_o *o, int64_t nsteps) /* the run loop body (E:6380-6386) */
{
    for (int64_t s = 0; s < nsteps; ++s) {
        o->klok += 1;
        deterministic_forces(o);
        full_forces(o);
        move(o);
        check_shifts(o);
    }
}

/* ---- set-up and accessors ------------------------------------------------ */
tis_o *tis_o_create(const tis_o_desc *d)
{
    tis_o *o = (tis_o *)calloc(1, sizeof(tis_o));
    o->d = *d;
    const int n = d->n;
    o->type = (int32_t *)dupm(d->type, sizeof(int32_t) * (size_t)n);
    o->kind = (int32_t *)dupm(d->kind, sizeof(int32_t) * (size_t)n);
    o->bt_kind = (int32_t *)dupm(d->bt_kind, sizeof(int32_t) * (size_t)d->n_bt);
    o->bt_a = (int32_t *)dupm(d->bt_a, sizeof(int32_t) * (size_t)d->n_bt);
    o->bt_b = (int32_t *)dupm(d->bt_b, sizeof(int32_t) * (size_t)d->n_bt);
    o->bt_c = (int32_t *)dupm(d->bt_c, sizeof(int32_t) * (size_t)d->n_bt);
    o->bt_k0 = (double *)dupm(d->bt_k0, sizeof(double) * (size_t)d->n_bt);
    o->bt_x0 = (double *)dupm(d->bt_x0, sizeof(double) * (size_t)d->n_bt);
    o->st3_idx = (int32_t *)dupm(d->st3_idx, sizeof(int32_t) * 6 * (size_t)d->n_st3);
    o->st3_off = (int32_t *)dupm(d->st3_off, sizeof(int32_t) * 2 * (size_t)d->n_st3);
    o->st3_native = (double *)dupm(d->st3_native, sizeof(double) * 6 * (size_t)d->n_st3);
    o->st3_E = (double *)dupm(d->st3_E, sizeof(double) * (size_t)d->n_st3);
    o->st2_idx = (int32_t *)dupm(d->st2_idx, sizeof(int32_t) * 7 * (size_t)d->n_st2);
    o->st2_r0 = (double *)dupm(d->st2_r0, sizeof(double) * (size_t)d->n_st2);
    o->st2_E = (double *)dupm(d->st2_E, sizeof(double) * (size_t)d->n_st2);
    o->hb_idx = (int32_t *)dupm(d->hb_idx, sizeof(int32_t) * 6 * (size_t)d->n_hb);
    o->hb_native = (double *)dupm(d->hb_native, sizeof(double) * 6 * (size_t)d->n_hb);
    o->hb_E = (double *)dupm(d->hb_E, sizeof(double) * (size_t)d->n_hb);
    o->hb_dode = (int32_t *)dupm(d->hb_dode, sizeof(int32_t) * (size_t)d->n_hb);
    o->hb_atom_off = (int32_t *)dupm(d->hb_atom_off, sizeof(int32_t) * ((size_t)d->n_hb + 1));
    o->hb_atom_idx = (int32_t *)dupm(d->hb_atom_idx, sizeof(int32_t) * (size_t)d->hb_atom_off[d->n_hb]);
    o->hba_valence = (int32_t *)dupm(d->hba_valence, sizeof(int32_t) * (size_t)d->n_hba);
    o->hba_cand_off = (int32_t *)dupm(d->hba_cand_off, sizeof(int32_t) * ((size_t)d->n_hba + 1));
    o->hba_cand_idx = (int32_t *)dupm(d->hba_cand_idx, sizeof(int32_t) * (size_t)d->hba_cand_off[d->n_hba]);
    o->d.type = o->type; o->d.kind = o->kind;

    /* parameter tables (read_maxi_key, E:2883-2945) */
    for (int t = 1; t <= NA; ++t) {
        double m = d->mass[t - 1], R = d->rlj[t - 1];
        o->MASS[t] = m;
        o->VISC[t] = 0.555 * R;
        o->K1[t] = exp(-o->VISC[t] / m * d->h);
        o->K2[t] = (1.0 - o->K1[t]) / o->VISC[t];
        o->SIGMA[t] = sqrt(2.0 * o->VISC[t] * d->T / d->h);
    }
    for (int a = 1; a <= NA; ++a)
        for (int b = a; b <= NA; ++b) {
            int J = jn12(a, b);
            o->D_LJ[J] = (a <= 6 && b <= 6) ? 3.2 : d->rlj[a - 1] + d->rlj[b - 1];
            o->D2_CUT[J] = o->D_LJ[J] * o->D_LJ[J];
            o->D2_MIN[J] = (o->D_LJ[J] - 0.4406141861 * SIG0) * (o->D_LJ[J] - 0.4406141861 * SIG0);
            o->E_LJ[J] = sqrt(d->elj[a - 1] * d->elj[b - 1]);
            o->F_LJ[J] = 12.0 * o->E_LJ[J] / (SIG0 * SIG0);
            o->Q_C[J] = d->qc[a - 1] * d->qc[b - 1];
        }
    o->hX = 0.5 * d->box[0]; o->hY = 0.5 * d->box[1]; o->hZ = 0.5 * d->box[2];
    o->D2_CT = d->rc * d->rc;
    o->R2_SR = (d->sr + d->skin) * (d->sr + d->skin);
    o->R2_LR = (d->rc + d->skin) * (d->rc + d->skin);

    double **st[15] = { &o->x, &o->y, &o->z, &o->xo, &o->yo, &o->zo, &o->vx, &o->vy, &o->vz,
                        &o->fx, &o->fy, &o->fz, &o->flx, &o->fly, &o->flz };
    for (int s = 0; s < 15; ++s) *st[s] = (double *)calloc((size_t)n + 1, sizeof(double));
    o->cell_of = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
    o->cell_list = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
    o->hb_status = (int32_t *)calloc((size_t)d->n_hb + 1, sizeof(int32_t));
    o->hb_energy = (double *)calloc((size_t)d->n_hb + 1, sizeof(double));
    o->hb_psi0 = (double *)calloc(3 * (size_t)d->n_hb + 3, sizeof(double));
    o->hb_K = (int32_t *)calloc((size_t)d->n_hb + 2, sizeof(int32_t));
    o->HB_EXCESS = (int32_t *)calloc((size_t)d->n_hba + 1, sizeof(int32_t));
    o->EXCESS = (int32_t *)calloc((size_t)d->n_hba + 1, sizeof(int32_t));
    o->hb_A = (int32_t *)calloc((size_t)d->n_hba + 2, sizeof(int32_t));
    o->HB_ATOM_N = (int32_t *)calloc((size_t)d->n_hba + 1, sizeof(int32_t));
    for (int a = 0; a < d->n_hba; ++a) o->HB_ATOM_N[a] = d->hba_cand_off[a + 1] - d->hba_cand_off[a];
    o->st_energy = (double *)calloc((size_t)(d->n_st3 + d->n_st2) + 1, sizeof(double));
    o->st_status = (int32_t *)calloc((size_t)(d->n_st3 + d->n_st2) + 1, sizeof(int32_t));
    /* HB_PAIR (E:4088-4107) as candidates sorted by central-pair key */
    {
        const int64_t NR = d->n_rna;
        int64_t *tmp = (int64_t *)malloc(sizeof(int64_t) * 2 * ((size_t)d->n_hb + 1));
        for (int k = 0; k < d->n_hb; ++k) {
            int a = d->hb_idx[6 * k + 1], b = d->hb_idx[6 * k + 4];
            int64_t key = a < b ? (int64_t)a * NR + b : (int64_t)b * NR + a;
            tmp[2 * k] = key;
            tmp[2 * k + 1] = k;
        }
        qsort(tmp, (size_t)d->n_hb, 2 * sizeof(int64_t), pair_key_cmp); /* ties keep no order; status is a set */
        o->pair_key = (int64_t *)malloc(sizeof(int64_t) * ((size_t)d->n_hb + 1));
        o->pair_cand = (int32_t *)malloc(sizeof(int32_t) * ((size_t)d->n_hb + 1));
        for (int k = 0; k < d->n_hb; ++k) { o->pair_key[k] = tmp[2 * k]; o->pair_cand[k] = (int32_t)tmp[2 * k + 1]; }
        free(tmp);
    }
    o->klok = 0;
    o->PROGRESS = 0;
    o->ctr = 0;
    return o;
}

void tis_o_destroy(tis_o *o)
{
    if (!o) return;
    void *ptrs[] = { o->type, o->kind, o->bt_kind, o->bt_a, o->bt_b, o->bt_c, o->bt_k0, o->bt_x0,
                     o->st3_idx, o->st3_off, o->st3_native, o->st3_E, o->st2_idx, o->st2_r0, o->st2_E,
                     o->hb_idx, o->hb_native, o->hb_E, o->hb_dode, o->hb_atom_off, o->hb_atom_idx,
                     o->hba_valence, o->hba_cand_off, o->hba_cand_idx, o->x, o->y, o->z, o->xo, o->yo, o->zo,
                     o->vx, o->vy, o->vz, o->fx, o->fy, o->fz, o->flx, o->fly, o->flz, o->cell_of,
                     o->cell_start, o->cell_list, o->sr.v, o->lr.v, o->hb_status, o->HB_EXCESS, o->EXCESS,
                     o->HB_ATOM_N, o->hb_A, o->hb_K, o->hb_energy, o->hb_psi0, o->pair_key, o->pair_cand,
                     o->st_energy, o->st_status };
    for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; ++i) free(ptrs[i]);
    free(o);
}

void tis_o_set_state(tis_o *o, const double *x, const double *y, const double *z,
                     const double *xo, const double *yo, const double *zo,
                     const double *vx, const double *vy, const double *vz)
{
    size_t b = sizeof(double) * (size_t)o->d.n;
    memcpy(o->x, x, b); memcpy(o->y, y, b); memcpy(o->z, z, b);
    memcpy(o->xo, xo, b); memcpy(o->yo, yo, b); memcpy(o->zo, zo, b);
    memcpy(o->vx, vx, b); memcpy(o->vy, vy, b); memcpy(o->vz, vz, b);
}

void tis_o_get_state(const tis_o *o, double *x, double *y, double *z,
                     double *xo, double *yo, double *zo, double *vx, double *vy, double *vz)
{
    size_t b = sizeof(double) * (size_t)o->d.n;
    memcpy(x, o->x, b); memcpy(y, o->y, b); memcpy(z, o->z, b);
    memcpy(xo, o->xo, b); memcpy(yo, o->yo, b); memcpy(zo, o->zo, b);
    memcpy(vx, o->vx, b); memcpy(vy, o->vy, b); memcpy(vz, o->vz, b);
}

void tis_o_get_cells(const tis_o *o, int32_t *cell, int32_t *dims)
{
    memcpy(cell, o->cell_of, sizeof(int32_t) * (size_t)o->d.n);
    dims[0] = o->McX; dims[1] = o->McY; dims[2] = o->McZ;
}

int64_t tis_o_get_pairs(const tis_o *o, int which, int32_t *out, int64_t cap)
{
    const ivec *l = which ? &o->lr : &o->sr;
    int64_t n = l->n < cap ? l->n : cap;
    if (out && n > 0) memcpy(out, l->v, sizeof(int32_t) * (size_t)n);
    return l->n;
}

void tis_o_get_hb(const tis_o *o, int32_t *status, int32_t *excess)
{
    memcpy(status, o->hb_status, sizeof(int32_t) * (size_t)o->d.n_hb);
    memcpy(excess, o->HB_EXCESS, sizeof(int32_t) * (size_t)o->d.n_hba);
}

static void copy_f(const tis_o *o, const double *a, const double *b, const double *c, double *out)
{
    if (!out) return;
    for (int i = 0; i < o->d.n; ++i) { out[3 * i] = a[i]; out[3 * i + 1] = b[i]; out[3 * i + 2] = c[i]; }
}

void tis_o_terms(tis_o *o, double *f_sr, double *f_lr, double *f_bonded, double *f_stack,
                 double *f_hb, double *e, int32_t *st_status_out)
{
    int n = o->d.n;
    double E[TIS_O_NE] = { 0 };
    zero3(o->fx, o->fy, o->fz, n);
    sr_forces(o, &E[TIS_O_E_LJ], &E[TIS_O_E_COUL_SR]);
    copy_f(o, o->fx, o->fy, o->fz, f_sr);
    zero3(o->flx, o->fly, o->flz, n);
    lr_forces(o, &E[TIS_O_E_COUL_LR]);
    copy_f(o, o->flx, o->fly, o->flz, f_lr);
    zero3(o->fx, o->fy, o->fz, n);
    double eb[3] = { 0, 0, 0 };
    bonded_forces(o, eb);
    E[TIS_O_E_BOND] = eb[0]; E[TIS_O_E_ANGLE] = eb[1]; E[TIS_O_E_EXCL] = eb[2];
    copy_f(o, o->fx, o->fy, o->fz, f_bonded);
    zero3(o->fx, o->fy, o->fz, n);
    o->E2_STACK = o->E3_STACK = 0;
    stacking(o);
    if (st_status_out) memcpy(st_status_out, o->st_status, sizeof(int32_t) * (size_t)(o->d.n_st3 + o->d.n_st2));
    copy_f(o, o->fx, o->fy, o->fz, f_stack);
    zero3(o->fx, o->fy, o->fz, n);
    o->E2_HB = o->E3_HB = 0;
    hydrogen_bonds(o);
    copy_f(o, o->fx, o->fy, o->fz, f_hb);
    E[TIS_O_E2_STACK] = o->E2_STACK; E[TIS_O_E3_STACK] = o->E3_STACK;
    E[TIS_O_E2_HB] = o->E2_HB; E[TIS_O_E3_HB] = o->E3_HB;
    E[TIS_O_RG] = radius_of_gyration(o);
    if (e) memcpy(e, E, sizeof E);
}

static int cmp_i64(const void *a, const void *b)
{
    const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return x < y ? -1 : x > y;
}

/* F_sr + F_bonded of tis_o_terms (SR_interactions_lists E:1783-1847 and
 * polymer_constraints E:2354-2520), summed with the LJ of each bonded pair
 * weighted by one minus the number of bonded terms that name it instead of added
 * in the pair sum and subtracted once per term (reduce_forces, E:880-897): the
 * same force in exact arithmetic, without the cancellation of the two equal
 * values, which loses the other pair forces of the bead when a folded 1-3 pair
 * makes them reach 1e17 and more. */
void tis_o_net_sr_bonded(tis_o *o, double *f)
{
    int n = o->d.n;
    int64_t *key = (int64_t *)malloc(sizeof(int64_t) * (size_t)(o->d.n_bt > 0 ? o->d.n_bt : 1));
    for (int t = 0; t < o->d.n_bt; ++t) {
        int a = o->bt_a[t], b = o->bt_kind[t] == 0 ? o->bt_b[t] : o->bt_c[t];
        int lo = a < b ? a : b, hi = a < b ? b : a;
        key[t] = (int64_t)lo * n + hi;
    }
    qsort(key, (size_t)o->d.n_bt, sizeof(int64_t), cmp_i64);
    zero3(o->fx, o->fy, o->fz, n);
    double v[3];
    for (int64_t p = 0; p < o->sr.n; p += 2) {
        int i = o->sr.v[p], j = o->sr.v[p + 1];
        int lo = i < j ? i : j, hi = i < j ? j : i;
        int64_t k = (int64_t)lo * n + hi;
        int mult = 0;
        const int64_t *hit = (const int64_t *)bsearch(&k, key, (size_t)o->d.n_bt, sizeof(int64_t), cmp_i64);
        if (hit) {
            const int64_t *a = hit, *b = hit;
            while (a > key && a[-1] == k) --a;
            while (b + 1 < key + o->d.n_bt && b[1] == k) ++b;
            mult = (int)(b - a) + 1;
        }
        int J = jn12(o->type[i], o->type[j]);
        double r2 = image_r2(o, i, j, v);
        double t = mult == 1 ? 0.0 : (1.0 - mult) * lj_force(o, r2, J);
        if (charged(o, i) && charged(o, j)) t += coulomb_force(o, r2, J);
        v[0] *= t; v[1] *= t; v[2] *= t;
        o->fx[i] += v[0]; o->fx[j] -= v[0];
        o->fy[i] += v[1]; o->fy[j] -= v[1];
        o->fz[i] += v[2]; o->fz[j] -= v[2];
    }
    free(key);
    for (int t = 0; t < o->d.n_bt; ++t) {
        int a = o->bt_a[t], b = o->bt_b[t], c = o->bt_c[t];
        if (o->bt_kind[t] == 0) bond_force(o, a, b, o->bt_k0[t], o->bt_x0[t]);
        else angle_force(o, a, b, c, o->bt_k0[t], o->bt_x0[t], 0);
    }
    copy_f(o, o->fx, o->fy, o->fz, f);
}

void tis_o_last_energies(const tis_o *o, double *out5)
{
    out5[0] = o->E2_HB; out5[1] = o->E3_HB; out5[2] = o->E2_STACK; out5[3] = o->E3_STACK;
    out5[4] = radius_of_gyration(o);
}

void tis_o_last_forces(const tis_o *o, double *f3n) { copy_f(o, o->fx, o->fy, o->fz, f3n); }
uint64_t tis_o_draws(const tis_o *o) { return o->ctr; }
int64_t tis_o_rebuilds(const tis_o *o) { return o->rebuilds; }
int64_t tis_o_klok(const tis_o *o) { return o->klok; }

/* one Philox-4x32-10 output word (for known-answer tests of the shared stream) */
uint32_t tis_o_philox_word(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, int lane)
{
    uint32_t c[4] = { c0, c1, c2, c3 };
    tis_o_philox4x32_10(c, k0, k1);
    return c[lane & 3];
}
