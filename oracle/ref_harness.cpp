/* TEST INFRASTRUCTURE — driver for the reference engine compiled as the CPU oracle.
 *
 * oracle/build_ref.py makes a build-time copy of src/16SCD_Mg_Cl_K_COPY_fast.cpp
 * (patch table in that script), compiles it with -Dmain=tis_ref_main, and links it
 * with this file.  Nothing here re-implements the physics: every force, energy,
 * list and step below is computed by the engine's own functions on its own
 * globals.  This file only
 *   - runs the engine's set-up sequence of main() (E:6038-6237) with parameters
 *     taken from the command line instead of compile-time literals,
 *   - exports the engine's arrays (0-based) to TISB files for the tests,
 *   - calls the hot-path functions on request.
 * E: = src/16SCD_Mg_Cl_K_COPY_fast.cpp of naotohori/16S-central-folding.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <vector>
#include <string>

#include "oracle_rng.h"
#include "tisb_io.h"

/* ---- engine globals (E:14-376) -------------------------------------------- */
extern long int klok;
extern int my_rank, comm_size;
extern double side_X, side_Y, side_Z, side_XYZ, side_hX, side_hY, side_hZ;
extern double h, T;
extern int NBP_atom, NB_atom, NTP_atom, NT_atom;
extern int **atom_key;
extern char *amino_key;
extern int *part_key, *maxi_key;
extern double MASS[], RLJ[], ELJ[], QC[], VISC[], K1[], K2[], SIGMA_FORCE[];
extern double D_LJ[], D2_LJ_MINIMUM[], E_LJ[], F_LJ[], Q_C[];
extern double cM_crwd[];
extern int N_crwd[];
extern double *x, *y, *z, *x_old, *y_old, *z_old, *vx, *vy, *vz;
extern double *fx, *fy, *fz, *flx, *fly, *flz, *fsend, *freceive;
extern int McX, McY, McZ, McT;
extern int **cell_content, *cell_mass;
extern int *list_content[];
extern int list_mass[];
extern double R1_LIST[], R2_LIST[];
extern double PROGRESS, dr1;
extern double st_D, ss_D;
extern int s3_N, st_N;
extern int *st_i, *st_j;
extern double *st_r, *st_theta1, *st_theta2, *st_psi, *st_psi1, *st_psi2, *st_E, *st_energy;
extern int *st_status, *ST_EXCESS;
extern int **ATOM_ST;
extern double hs_D;
extern int hb_N;
extern int *hb_dode, *hb_k10, *hb_k11, *hb_k12, *hb_k20, *hb_k21, *hb_k22;
extern double *hb_r, *hb_theta1, *hb_theta2, *hb_psi, *hb_psi1, *hb_psi2, *hb_E, *hb_energy;
extern int *hb_status;
extern int HB_NT_atom;
extern int *VALENCE, *HB_EXCESS, *HB_ATOM_N, **HB_ATOM, *ATOM_HB_N, **ATOM_HB;
extern double lB, D_CT_CUTOFF, D2_CT_CUTOFF;
extern double E2_HB, E3_HB, E2_STACK, E3_STACK, ELJ_NON_NATIVE;

/* ---- engine functions ---------------------------------------------------- */
void read_maxi_key(char *);
void list_crowder_types(void);
void read_PDB(char *);
void initialize_HB_atoms(void);
void initialize_unprocessed_bonds(char *);
void initialize_unprocessed_stacks(char *);
void set_box(int);
void add_crowder(int);
void populate_lists(void);
void check_shifts(void);
void SR_interactions_lists(void);
void LR_interactions_lists(void);
void stacking_interactions(void);
void hydrogen_bonds_interactions(void);
void polymer_constraints(void);
void deterministic_forces_MPI(void);
void full_forces(void);
void move_rigid_units(void);
double radius_of_gyration(int, int);
double WCA_ENERGY(double, int);
double COULOMB_TRUNCATED_ENERGY(double, int);
void CC_energy_single_pair(int, int, int, double, double (*)(double, int), double *);
void reduce_energies(int, int, double);
double CC_distance(int, int);
double valence_angle(int, int, int);
void half_shift(double *);

/* ---- patched-in symbols (see tis_ref_hooks.h) ---------------------------- */
int tis_center_atom = 500;

static int g_record = 0;      /* 1: record bonded terms; 2: accumulate bonded energies */
struct BondedTerm { int kind, a, b, c; double k0, x0; };
static std::vector<BondedTerm> g_terms;
static double g_e_bond = 0, g_e_angle = 0;

void tis_hook_bond(int i1, int i2, double k0, double r0)
{
    if (g_record == 1) g_terms.push_back({0, i1 - 1, i2 - 1, -1, k0, r0});
    if (g_record == 2) {
        double r = CC_distance(i1, i2);
        g_e_bond += k0 * (r - r0) * (r - r0);
        reduce_energies(i1, i2, -1.0); /* the engine's own WCA energy of the excluded pair */
    }
}

void tis_hook_angle(int i1, int i2, int i3, double k0, double theta0)
{
    if (g_record == 1) g_terms.push_back({1, i1 - 1, i2 - 1, i3 - 1, k0, theta0});
    if (g_record == 2) {
        double t = valence_angle(i1, i2, i3);
        g_e_angle += k0 * (t - theta0) * (t - theta0);
        reduce_energies(i1, i3, -1.0);
    }
}

/* ---- rand()/srand() shim ------------------------------------------------- */
/* This translation unit is compiled WITHOUT ref_rng_shim.h, so rand()/srand()
 * below are glibc's own. */
static int g_rng_philox = 0;
static uint64_t g_seed = 1, g_ctr = 0;

extern "C" int tis_shim_rand(void)
{
    if (!g_rng_philox) return rand();
    return tis_o_rand_value(g_seed, 0u, g_ctr++);
}

extern "C" void tis_shim_srand(unsigned s)
{
    if (!g_rng_philox) srand(s);
}

/* ---- TISB state reader --------------------------------------------------- */
static int read_state_file(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "tis_ref: cannot open %s\n", path); return 1; }
    char magic[8];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "TISB0001", 8) != 0) { fclose(f); return 2; }
    double **dst[9] = { &x, &y, &z, &x_old, &y_old, &z_old, &vx, &vy, &vz };
    const char *names[9] = { "x", "y", "z", "x_old", "y_old", "z_old", "vx", "vy", "vz" };
    int found = 0;
    for (;;) {
        char nm[32], dt[4]; int64_t n;
        if (fread(nm, 1, 32, f) != 32) break;
        if (fread(dt, 1, 4, f) != 4 || fread(&n, 8, 1, f) != 1) break;
        size_t es = (dt[0] == 'f' || dt[1] == '8') ? 8 : 4;
        std::vector<char> buf((size_t)n * es);
        if (n > 0 && fread(buf.data(), es, (size_t)n, f) != (size_t)n) break;
        for (int a = 0; a < 9; ++a) {
            if (strcmp(nm, names[a]) == 0 && dt[0] == 'f' && n == NT_atom) {
                const double *src = (const double *)buf.data();
                for (int i = 0; i < NT_atom; ++i) (*dst[a])[i + 1] = src[i];
                found |= 1 << a;
            }
        }
    }
    fclose(f);
    return (found & 7) == 7 ? 0 : 3;
}

/* ---- exports --------------------------------------------------------------- */
static void put_particles(FILE *f, const char *px, double *a, double *b, double *c)
{
    std::vector<double> t(NT_atom);
    const char *sfx[3] = { "x", "y", "z" };
    double *arr[3] = { a, b, c };
    for (int d = 0; d < 3; ++d) {
        for (int i = 0; i < NT_atom; ++i) t[i] = arr[d][i + 1];
        std::string nm = std::string(px) + sfx[d];
        tisb_put_f8(f, nm.c_str(), t.data(), NT_atom);
    }
}

static void put_state(FILE *f)
{
    put_particles(f, "", x, y, z);
    put_particles(f, "o", x_old, y_old, z_old);
    put_particles(f, "v", vx, vy, vz);
}

static void zero_forces(void)
{
    for (int i = 0; i <= NT_atom; ++i) { fx[i] = fy[i] = fz[i] = 0; }
}

static void put_forces(FILE *f, const char *name, double *a, double *b, double *c)
{
    std::vector<double> t(3 * (size_t)NT_atom);
    for (int i = 0; i < NT_atom; ++i) { t[3 * i] = a[i + 1]; t[3 * i + 1] = b[i + 1]; t[3 * i + 2] = c[i + 1]; }
    tisb_put_f8(f, name, t.data(), 3 * (int64_t)NT_atom);
}

static void export_system(const char *path)
{
    FILE *f = tisb_open_write(path);
    if (!f) { fprintf(stderr, "tis_ref: cannot write %s\n", path); exit(2); }
    tisb_put_scalar_i8(f, "n_particles", NT_atom);
    tisb_put_scalar_i8(f, "n_rna", NTP_atom);
    tisb_put_scalar_i8(f, "n_entries", NBP_atom);
    tisb_put_scalar_i8(f, "center", tis_center_atom - 1);
    double box[3] = { side_X, side_Y, side_Z };
    tisb_put_f8(f, "box", box, 3);
    tisb_put_scalar_f8(f, "T", T);
    tisb_put_scalar_f8(f, "h", h);
    tisb_put_scalar_f8(f, "lB", lB);
    tisb_put_scalar_f8(f, "rc", D_CT_CUTOFF);
    tisb_put_scalar_f8(f, "ss_D", ss_D);
    tisb_put_scalar_f8(f, "hs_D", hs_D);
    tisb_put_scalar_f8(f, "st_D", st_D);
    int32_t nion[3] = { N_crwd[0], N_crwd[1], N_crwd[2] };
    tisb_put_i4(f, "n_ions", nion, 3); /* Mg, Cl, K (crowder types 0,1,2; E:2960-3130) */

    std::vector<int32_t> ti(NT_atom), ki(NT_atom);
    for (int i = 0; i < NT_atom; ++i) { ti[i] = maxi_key[i + 1]; ki[i] = part_key[i + 1]; }
    tisb_put_i4(f, "type", ti.data(), NT_atom);
    tisb_put_i4(f, "kind", ki.data(), NT_atom);
    tisb_put_f8(f, "mass", MASS + 1, 9);
    tisb_put_f8(f, "rlj", RLJ + 1, 9);
    tisb_put_f8(f, "elj", ELJ + 1, 9);
    tisb_put_f8(f, "qc", QC + 1, 9);

    std::vector<int32_t> ec(NBP_atom), e0(NBP_atom), e1(NBP_atom);
    for (int e = 1; e <= NBP_atom; ++e) {
        ec[e - 1] = amino_key[e];
        e0[e - 1] = atom_key[e][0] - 1;
        e1[e - 1] = (amino_key[e] == 'P') ? -1 : atom_key[e][1] - 1;
    }
    tisb_put_i4(f, "entry_code", ec.data(), NBP_atom);
    tisb_put_i4(f, "entry_a0", e0.data(), NBP_atom);
    tisb_put_i4(f, "entry_a1", e1.data(), NBP_atom);

    /* bonded terms exactly as the engine's polymer_constraints() visits them */
    g_terms.clear();
    g_record = 1;
    zero_forces();
    polymer_constraints();
    zero_forces();
    g_record = 0;
    {
        size_t n = g_terms.size();
        std::vector<int32_t> kd(n), a(n), b(n), c(n);
        std::vector<double> k0(n), x0(n);
        for (size_t t = 0; t < n; ++t) {
            kd[t] = g_terms[t].kind; a[t] = g_terms[t].a; b[t] = g_terms[t].b; c[t] = g_terms[t].c;
            k0[t] = g_terms[t].k0; x0[t] = g_terms[t].x0;
        }
        tisb_put_i4(f, "bt_kind", kd.data(), n);
        tisb_put_i4(f, "bt_a", a.data(), n);
        tisb_put_i4(f, "bt_b", b.data(), n);
        tisb_put_i4(f, "bt_c", c.data(), n);
        tisb_put_f8(f, "bt_k0", k0.data(), n);
        tisb_put_f8(f, "bt_x0", x0.data(), n);
    }

    /* tertiary stacks: particle sextets as stacking_interactions() forms them (E:1932-1948) */
    {
        int n = s3_N;
        std::vector<int32_t> idx(6 * (size_t)n), site(2 * (size_t)n), si(n), sj(n);
        std::vector<double> nat(6 * (size_t)n), E(n);
        for (int k = 1; k <= n; ++k) {
            int i = st_i[k], j = st_j[k];
            si[k - 1] = i; sj[k - 1] = j;
            idx[6 * (k - 1) + 0] = atom_key[i][0] - 1;
            idx[6 * (k - 1) + 1] = atom_key[i][1] - 1;
            idx[6 * (k - 1) + 2] = atom_key[i + 1][0] - 1;
            idx[6 * (k - 1) + 3] = atom_key[j][0] - 1;
            idx[6 * (k - 1) + 4] = atom_key[j][1] - 1;
            idx[6 * (k - 1) + 5] = atom_key[j + 1][0] - 1;
            nat[6 * (k - 1) + 0] = st_r[k]; nat[6 * (k - 1) + 1] = st_theta1[k];
            nat[6 * (k - 1) + 2] = st_theta2[k]; nat[6 * (k - 1) + 3] = st_psi[k];
            nat[6 * (k - 1) + 4] = st_psi1[k]; nat[6 * (k - 1) + 5] = st_psi2[k];
            E[k - 1] = st_E[k];
            site[2 * (k - 1)] = ATOM_ST[k][0]; site[2 * (k - 1) + 1] = ATOM_ST[k][1];
        }
        tisb_put_i4(f, "st3_entry_i", si.data(), n);
        tisb_put_i4(f, "st3_entry_j", sj.data(), n);
        tisb_put_i4(f, "st3_idx", idx.data(), 6 * (int64_t)n);
        tisb_put_f8(f, "st3_native", nat.data(), 6 * (int64_t)n);
        tisb_put_f8(f, "st3_E", E.data(), n);
        tisb_put_i4(f, "st3_site", site.data(), 2 * (int64_t)n);
        std::vector<int32_t> ex(NBP_atom);
        for (int e = 1; e <= NBP_atom; ++e) ex[e - 1] = ST_EXCESS[e];
        tisb_put_i4(f, "st_excess", ex.data(), NBP_atom);
    }
    /* secondary stacks (E:2069-2084) */
    {
        int n = st_N - s3_N;
        std::vector<int32_t> idx(7 * (size_t)n), si(n);
        std::vector<double> r0(n), E(n);
        for (int k = s3_N + 1; k <= st_N; ++k) {
            int i = st_i[k], t = k - s3_N - 1;
            si[t] = i;
            idx[7 * t + 0] = atom_key[i - 1][0] - 1;
            idx[7 * t + 1] = atom_key[i][0] - 1;
            idx[7 * t + 2] = atom_key[i][1] - 1;
            idx[7 * t + 3] = atom_key[i + 1][0] - 1;
            idx[7 * t + 4] = atom_key[i + 2][0] - 1;
            idx[7 * t + 5] = atom_key[i + 2][1] - 1;
            idx[7 * t + 6] = atom_key[i + 3][0] - 1;
            r0[t] = st_r[k]; E[t] = st_E[k];
        }
        tisb_put_i4(f, "st2_entry_i", si.data(), n);
        tisb_put_i4(f, "st2_idx", idx.data(), 7 * (int64_t)n);
        tisb_put_f8(f, "st2_r0", r0.data(), n);
        tisb_put_f8(f, "st2_E", E.data(), n);
    }
    /* hydrogen-bond candidates and valence tables (E:3733-4119, E:3671-3729) */
    {
        int n = hb_N;
        std::vector<int32_t> idx(6 * (size_t)n), dode(n), aoff(n + 1);
        std::vector<double> nat(6 * (size_t)n), E(n);
        std::vector<int32_t> alist;
        aoff[0] = 0;
        for (int k = 1; k <= n; ++k) {
            int t = k - 1;
            idx[6 * t + 0] = hb_k10[k] - 1; idx[6 * t + 1] = hb_k11[k] - 1; idx[6 * t + 2] = hb_k12[k] - 1;
            idx[6 * t + 3] = hb_k20[k] - 1; idx[6 * t + 4] = hb_k21[k] - 1; idx[6 * t + 5] = hb_k22[k] - 1;
            nat[6 * t + 0] = hb_r[k]; nat[6 * t + 1] = hb_theta1[k]; nat[6 * t + 2] = hb_theta2[k];
            nat[6 * t + 3] = hb_psi[k]; nat[6 * t + 4] = hb_psi1[k]; nat[6 * t + 5] = hb_psi2[k];
            E[t] = hb_E[k]; dode[t] = hb_dode[k];
            for (int a = 1; a <= ATOM_HB_N[k]; ++a) alist.push_back(ATOM_HB[k][a] - 1);
            aoff[k] = (int32_t)alist.size();
        }
        tisb_put_i4(f, "hb_idx", idx.data(), 6 * (int64_t)n);
        tisb_put_f8(f, "hb_native", nat.data(), 6 * (int64_t)n);
        tisb_put_f8(f, "hb_E", E.data(), n);
        tisb_put_i4(f, "hb_dode", dode.data(), n);
        tisb_put_i4(f, "hb_atom_off", aoff.data(), n + 1);
        tisb_put_i4(f, "hb_atom_idx", alist.data(), (int64_t)alist.size());
        int na = HB_NT_atom;
        std::vector<int32_t> val(na), coff(na + 1), clist;
        coff[0] = 0;
        for (int a = 1; a <= na; ++a) {
            val[a - 1] = VALENCE[a];
            for (int j = 1; j <= HB_ATOM_N[a]; ++j) clist.push_back(HB_ATOM[a][j] - 1);
            coff[a] = (int32_t)clist.size();
        }
        tisb_put_i4(f, "hba_valence", val.data(), na);
        tisb_put_i4(f, "hba_cand_off", coff.data(), na + 1);
        tisb_put_i4(f, "hba_cand_idx", clist.data(), (int64_t)clist.size());
    }
    put_state(f);
    fclose(f);
}

static void export_lists(const char *path)
{
    FILE *f = tisb_open_write(path);
    int32_t mc[3] = { McX, McY, McZ };
    tisb_put_i4(f, "cells_dim", mc, 3);
    std::vector<int32_t> cell(NT_atom, -1);
    for (int m = 1; m <= McT; ++m)
        for (int j = 1; j <= cell_mass[m]; ++j) cell[cell_content[m][j] - 1] = m - 1;
    tisb_put_i4(f, "cell", cell.data(), NT_atom);
    for (int L = 0; L < 2; ++L) {
        std::vector<int32_t> pr((size_t)list_mass[L]);
        for (int k = 1; k <= list_mass[L]; ++k) pr[k - 1] = list_content[L][k] - 1;
        tisb_put_i4(f, L == 0 ? "sr_pairs" : "lr_pairs", pr.data(), list_mass[L]);
    }
    std::vector<int32_t> st(hb_N), ex(HB_NT_atom);
    for (int k = 1; k <= hb_N; ++k) st[k - 1] = hb_status[k];
    for (int a = 1; a <= HB_NT_atom; ++a) ex[a - 1] = HB_EXCESS[a];
    tisb_put_i4(f, "hb_status", st.data(), hb_N);
    tisb_put_i4(f, "hb_excess", ex.data(), HB_NT_atom);
    fclose(f);
}

static int jn12(int i, int j)
{
    int a = maxi_key[i], b = maxi_key[j];
    if (a < b) return (a - 1) * 9 - (a - 1) * a / 2 + b;
    return (b - 1) * 9 - (b - 1) * b / 2 + a;
}

/* Per-term forces and energies on the current state, each term evaluated by the
 * engine's own function into zeroed force arrays. */
static void export_terms(const char *path)
{
    FILE *f = tisb_open_write(path);
    zero_forces();
    SR_interactions_lists();
    put_forces(f, "F_sr", fx, fy, fz);
    for (int i = 0; i <= NT_atom; ++i) { flx[i] = fly[i] = flz[i] = 0; }
    LR_interactions_lists();
    put_forces(f, "F_lr", flx, fly, flz);
    zero_forces();
    polymer_constraints();
    put_forces(f, "F_bonded", fx, fy, fz);
    zero_forces();
    E2_STACK = E3_STACK = 0;
    stacking_interactions();
    put_forces(f, "F_stack", fx, fy, fz);
    tisb_put_scalar_f8(f, "E2_STACK", E2_STACK);
    tisb_put_scalar_f8(f, "E3_STACK", E3_STACK);
    {
        std::vector<double> se(st_N);
        std::vector<int32_t> ss(st_N);
        for (int k = 1; k <= st_N; ++k) { se[k - 1] = st_energy[k]; ss[k - 1] = st_status[k]; }
        tisb_put_f8(f, "st_energy", se.data(), st_N);
        tisb_put_i4(f, "st_status", ss.data(), st_N);
    }
    zero_forces();
    E2_HB = E3_HB = 0;
    uint64_t ctr0 = g_ctr;
    hydrogen_bonds_interactions();
    put_forces(f, "F_hb", fx, fy, fz);
    tisb_put_scalar_f8(f, "E2_HB", E2_HB);
    tisb_put_scalar_f8(f, "E3_HB", E3_HB);
    tisb_put_scalar_i8(f, "hb_draws", (int64_t)(g_ctr - ctr0));
    {
        std::vector<double> he(hb_N);
        for (int k = 1; k <= hb_N; ++k) he[k - 1] = hb_energy[k];
        tisb_put_f8(f, "hb_energy", he.data(), hb_N);
    }
    /* pair energies over the engine's lists with the engine's energy functions */
    double e_lj = 0, e_csr = 0, e_clr = 0;
    for (int k = 1; k <= list_mass[0]; k += 2) {
        int i = list_content[0][k], j = list_content[0][k + 1], J = jn12(i, j);
        CC_energy_single_pair(i, j, J, 1.0, WCA_ENERGY, &e_lj);
        if (part_key[i] != 1 && part_key[i] != 2 && part_key[j] != 1 && part_key[j] != 2)
            CC_energy_single_pair(i, j, J, 1.0, COULOMB_TRUNCATED_ENERGY, &e_csr);
    }
    for (int k = 1; k <= list_mass[1]; k += 2) {
        int i = list_content[1][k], j = list_content[1][k + 1], J = jn12(i, j);
        CC_energy_single_pair(i, j, J, 1.0, COULOMB_TRUNCATED_ENERGY, &e_clr);
    }
    tisb_put_scalar_f8(f, "E_lj", e_lj);
    tisb_put_scalar_f8(f, "E_coul_sr", e_csr);
    tisb_put_scalar_f8(f, "E_coul_lr", e_clr);
    g_e_bond = g_e_angle = 0; ELJ_NON_NATIVE = 0;
    g_record = 2;
    zero_forces();
    polymer_constraints();
    zero_forces();
    g_record = 0;
    tisb_put_scalar_f8(f, "E_bond", g_e_bond);
    tisb_put_scalar_f8(f, "E_angle", g_e_angle);
    tisb_put_scalar_f8(f, "E_excl", ELJ_NON_NATIVE);
    tisb_put_scalar_f8(f, "Rg", radius_of_gyration(1, NTP_atom));
    fclose(f);
}

/* ---- command line -------------------------------------------------------- */
static const char *arg_str(int argc, char **argv, const char *key, const char *def)
{
    for (int i = 1; i + 1 < argc; ++i) if (strcmp(argv[i], key) == 0) return argv[i + 1];
    return def;
}
static int has_flag(int argc, char **argv, const char *key)
{
    for (int i = 1; i < argc; ++i) if (strcmp(argv[i], key) == 0) return 1;
    return 0;
}

int main(int argc, char **argv)
{
    const char *pdb = arg_str(argc, argv, "--pdb", NULL);
    const char *bonds = arg_str(argc, argv, "--bonds", NULL);
    const char *stacks = arg_str(argc, argv, "--stacks", NULL);
    const char *maxikey = arg_str(argc, argv, "--maxikey", NULL);
    if (!pdb || !bonds || !stacks || !maxikey) {
        fprintf(stderr, "usage: tis_ref --pdb F --bonds F --stacks F --maxikey F [options]\n");
        return 2;
    }
    double box = atof(arg_str(argc, argv, "--box", "350"));
    T = atof(arg_str(argc, argv, "--T", "0.615"));
    ss_D = atof(arg_str(argc, argv, "--ssD", "0.850"));
    hs_D = atof(arg_str(argc, argv, "--hsD", "3.975"));
    st_D = atof(arg_str(argc, argv, "--stD", "6.5"));
    int seed = atoi(arg_str(argc, argv, "--seed", "1"));
    D_CT_CUTOFF = atof(arg_str(argc, argv, "--rc", "50"));
    D2_CT_CUTOFF = D_CT_CUTOFF * D_CT_CUTOFF;
    double sr = atof(arg_str(argc, argv, "--sr", "12"));
    double skin = atof(arg_str(argc, argv, "--skin", "3"));
    cM_crwd[0] = atof(arg_str(argc, argv, "--cMg", "0.005"));
    cM_crwd[2] = atof(arg_str(argc, argv, "--cK", "0.050"));
    tis_center_atom = atoi(arg_str(argc, argv, "--center", "500"));
    g_rng_philox = strcmp(arg_str(argc, argv, "--rng", "glibc"), "philox") == 0;
    g_seed = (uint64_t)seed;
    my_rank = 0; comm_size = 1;
    side_X = side_Y = side_Z = box;

    srand((unsigned)(T * 1000 * seed)); /* E:6105 (glibc mode only) */
    lB = 332.0637090 * (0.03273600947 * T - 0.00669625750); /* E:6109 */

    read_maxi_key((char *)maxikey);
    if (has_flag(argc, argv, "--no-noise")) for (int t = 1; t <= 9; ++t) SIGMA_FORCE[t] = 0;
    list_crowder_types();
    read_PDB((char *)pdb);
    initialize_HB_atoms();
    initialize_unprocessed_bonds((char *)bonds);
    initialize_unprocessed_stacks((char *)stacks);
    if (tis_center_atom < 1 || tis_center_atom > NTP_atom) {
        fprintf(stderr, "tis_ref: centre atom %d outside the RNA (1..%d)\n", tis_center_atom, NTP_atom);
        return 3;
    }
    set_box(tis_center_atom);
    if (arg_str(argc, argv, "--nMg", NULL)) {
        N_crwd[0] = atoi(arg_str(argc, argv, "--nMg", "0"));
        N_crwd[1] = atoi(arg_str(argc, argv, "--nCl", "0"));
        N_crwd[2] = atoi(arg_str(argc, argv, "--nK", "0"));
    } else { /* E:6167-6171 */
        N_crwd[0] = (int)(cM_crwd[0] * 6.022 * 0.0001 * side_XYZ);
        N_crwd[2] = (int)(cM_crwd[2] * 6.022 * 0.0001 * side_XYZ);
        N_crwd[1] = 2 * N_crwd[0] + N_crwd[2] - (NBP_atom - 1) / 2;
    }
    for (int t = 0; t < 3; ++t)
        for (int n = 1; n <= N_crwd[t]; ++n) add_crowder(t);

    fsend = (double *)calloc(3 * (size_t)NT_atom, sizeof(double));
    freceive = (double *)calloc(3 * (size_t)NT_atom, sizeof(double));
    dr1 = skin;
    R1_LIST[0] = sr + dr1; R2_LIST[0] = R1_LIST[0] * R1_LIST[0];
    R1_LIST[1] = D_CT_CUTOFF + dr1; R2_LIST[1] = R1_LIST[1] * R1_LIST[1];
    /* capacity: every pair of the system fits (the engine's 100000/500000 are E:6233-6235) */
    size_t cap = (size_t)NT_atom * (size_t)(NT_atom - 1) + 16;
    size_t cap_max = (size_t)NT_atom * 1200 + 16;
    if (cap > cap_max) cap = cap_max;
    list_content[0] = (int *)calloc(cap + 1, sizeof(int));
    list_content[1] = (int *)calloc(cap + 1, sizeof(int));

    if (arg_str(argc, argv, "--state-in", NULL)) {
        int rc = read_state_file(arg_str(argc, argv, "--state-in", NULL));
        if (rc) { fprintf(stderr, "tis_ref: bad state file (%d)\n", rc); return 4; }
    }
    g_ctr = 0; /* the step loop starts at draw 0 of the Philox stream */

    if (arg_str(argc, argv, "--export-system", NULL)) export_system(arg_str(argc, argv, "--export-system", NULL));

    populate_lists();
    PROGRESS = 0;
    if ((size_t)list_mass[0] > cap || (size_t)list_mass[1] > cap) {
        fprintf(stderr, "tis_ref: list capacity exceeded\n");
        return 5;
    }
    if (arg_str(argc, argv, "--lists", NULL)) export_lists(arg_str(argc, argv, "--lists", NULL));
    if (arg_str(argc, argv, "--terms", NULL)) {
        export_terms(arg_str(argc, argv, "--terms", NULL));
        g_ctr = 0;
    }

    long nsteps = atol(arg_str(argc, argv, "--steps", "0"));
    if (nsteps > 0) {
        long every = atol(arg_str(argc, argv, "--every", "0"));
        const char *traj = arg_str(argc, argv, "--traj", NULL);
        FILE *ft = traj ? tisb_open_write(traj) : NULL;
        std::vector<double> ener;
        std::vector<int32_t> rebuilds;
        struct timespec t0, t1;
        clock_gettime(CLOCK_MONOTONIC, &t0);
        for (klok = 1; klok <= nsteps; ++klok) {
            deterministic_forces_MPI();
            full_forces();
            move_rigid_units();
            check_shifts();
            if (PROGRESS == 0) rebuilds.push_back((int32_t)klok);
            if (ft && every > 0 && klok % every == 0) {
                char nm[32];
                std::vector<double> fr(3 * (size_t)NT_atom);
                for (int i = 0; i < NT_atom; ++i) { fr[3 * i] = x[i + 1]; fr[3 * i + 1] = y[i + 1]; fr[3 * i + 2] = z[i + 1]; }
                snprintf(nm, sizeof nm, "pos_%ld", klok);
                tisb_put_f8(ft, nm, fr.data(), 3 * (int64_t)NT_atom);
                double e[5] = { E2_HB, E3_HB, E2_STACK, E3_STACK, radius_of_gyration(1, NTP_atom) };
                ener.insert(ener.end(), e, e + 5);
            }
        }
        clock_gettime(CLOCK_MONOTONIC, &t1);
        double secs = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
        if (ft) {
            tisb_put_f8(ft, "energies", ener.data(), (int64_t)ener.size());
            tisb_put_i4(ft, "rebuild_steps", rebuilds.data(), (int64_t)rebuilds.size());
            tisb_put_scalar_i8(ft, "draws", (int64_t)g_ctr);
            put_state(ft);
            fclose(ft);
        }
        if (has_flag(argc, argv, "--time"))
            printf("{\"steps\": %ld, \"seconds\": %.6f, \"steps_per_s\": %.3f, \"n_particles\": %d}\n",
                   nsteps, secs, nsteps / secs, NT_atom);
    }
    return 0;
}
