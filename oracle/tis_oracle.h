/* TEST INFRASTRUCTURE — FP64 CPU oracle of the TIS-RNA Langevin step.
 *
 * A restatement, in plain C, of the per-step hot path of the reference engine
 * (src/16SCD_Mg_Cl_K_COPY_fast.cpp of naotohori/16S-central-folding, cited as E:),
 * used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * as the checker.  Never part of the product path.
 *
 * All indices are 0-based particle indices; the reference's 1-based arrays are
 * shifted by one.  The system arrays follow the names of the TISB system export
 * (oracle/ref_harness.cpp, export_system). */
#ifndef TIS_ORACLE_H
#define TIS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tis_o_desc {
    int32_t n, n_rna, center;            /* particles, RNA beads, recentring bead */
    double box[3];
    double T, h, lB, rc;                 /* temperature (kcal/mol), step, Bjerrum length, Coulomb cutoff */
    double sr, skin;                     /* SR list radius = sr + skin; LR radius = rc + skin */
    int32_t lr_interval;                 /* LR Coulomb refresh period (E:2550: 10) */
    uint64_t seed;                       /* Philox key of the rand() stream */
    int32_t noise;                       /* 1: Langevin noise on (E:2590), 0: off */
    const int32_t *type, *kind;          /* maxi_key 1..9, part_key 0..5 */
    const double *mass, *rlj, *elj, *qc; /* 9 entries each (MAXIKEY) */
    int32_t n_bt;                        /* bonded terms in polymer_constraints() order */
    const int32_t *bt_kind, *bt_a, *bt_b, *bt_c;
    const double *bt_k0, *bt_x0;
    int32_t n_st3;                       /* tertiary stacks */
    const int32_t *st3_idx;              /* 6 per stack: k10 k11 k12 k20 k21 k22 */
    const double *st3_native, *st3_E;    /* 6 per stack: r theta1 theta2 psi psi1 psi2 */
    const int32_t *st3_off;              /* 2 per stack: secondary stack switched off, or -1 */
    int32_t n_st2;                       /* secondary stacks */
    const int32_t *st2_idx;              /* 7 per stack: k_10 k00 k01 k10 k20 k21 k30 */
    const double *st2_r0, *st2_E;
    int32_t n_hb;                        /* hydrogen-bond candidates */
    const int32_t *hb_idx;               /* 6 per candidate */
    const double *hb_native, *hb_E;
    const int32_t *hb_dode, *hb_atom_off, *hb_atom_idx;
    int32_t n_hba;                       /* hydrogen-bonding atoms */
    const int32_t *hba_valence, *hba_cand_off, *hba_cand_idx;
    double debye;                        /* Debye length of the screened Coulomb term, A (0: unscreened,
                                            the reference's truncated Coulomb) */
} tis_o_desc;

typedef struct tis_o tis_o;

/* energies vector layout */
enum {
    TIS_O_E_LJ = 0, TIS_O_E_COUL_SR, TIS_O_E_COUL_LR, TIS_O_E_BOND, TIS_O_E_ANGLE, TIS_O_E_EXCL,
    TIS_O_E2_STACK, TIS_O_E3_STACK, TIS_O_E2_HB, TIS_O_E3_HB, TIS_O_RG, TIS_O_NE
};

tis_o *tis_o_create(const tis_o_desc *d);
void tis_o_destroy(tis_o *o);
void tis_o_set_state(tis_o *o, const double *x, const double *y, const double *z,
                     const double *xo, const double *yo, const double *zo,
                     const double *vx, const double *vy, const double *vz);
void tis_o_get_state(const tis_o *o, double *x, double *y, double *z,
                     double *xo, double *yo, double *zo, double *vx, double *vy, double *vz);
int tis_o_populate_lists(tis_o *o);
void tis_o_get_cells(const tis_o *o, int32_t *cell, int32_t *dims);
int64_t tis_o_get_pairs(const tis_o *o, int which, int32_t *out, int64_t cap);
void tis_o_get_hb(const tis_o *o, int32_t *status, int32_t *excess);
/* per-term forces (3n each, may be NULL) and energies (TIS_O_NE) on the current state */
void tis_o_terms(tis_o *o, double *f_sr, double *f_lr, double *f_bonded, double *f_stack,
                 double *f_hb, double *energies, int32_t *st_status);
/* F_sr + F_bonded with each bonded pair's LJ weighted in the pair sum instead of
 * added and subtracted (3n; see tis_oracle.c) */
void tis_o_net_sr_bonded(tis_o *o, double *f);
void tis_o_step(tis_o *o, int64_t nsteps);
/* E2_HB, E3_HB, E2_STACK, E3_STACK, Rg of the last step */
void tis_o_last_energies(const tis_o *o, double *out5);
uint64_t tis_o_draws(const tis_o *o);
int64_t tis_o_rebuilds(const tis_o *o);
int64_t tis_o_klok(const tis_o *o);
void tis_o_last_forces(const tis_o *o, double *f3n);

#ifdef __cplusplus
}
#endif
#endif
