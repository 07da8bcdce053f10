/* Declarations inserted by oracle/build_ref.py into the build-time copy of the
 * reference engine (TEST INFRASTRUCTURE).  The hooks record every bond and
 * valence term that the engine's own polymer_constraints() evaluates
 * (src/16SCD_Mg_Cl_K_COPY_fast.cpp:924, :1031), so the exported bonded-term list
 * is the one the reference actually uses; tis_center_atom replaces the literal
 * 500 of adjust_box(500) (:2670). */
#ifndef TIS_REF_HOOKS_H
#define TIS_REF_HOOKS_H
void tis_hook_bond(int i1, int i2, double k0, double r0);
void tis_hook_angle(int i1, int i2, int i3, double k0, double theta0);
extern int tis_center_atom;
#endif
