// Kernel interface of the TIS engine: device pointer bundle and launchers.
#pragma once
#include <cuda_runtime.h>

#include "tis_device.cuh"

namespace tis {

// Frames written from inside the step (tis_frames_start): every `every` steps the
// integrator's last block of each replica writes the replica's positions, its five
// Energies-file values and then its step number into a ring of `depth` slots in
// pinned, device-mapped host memory (every = 0: off).
struct FrameRing {
    double *pos;        // depth slots of 3 x n_total doubles: x, y, z of every replica end to end
    double *en;         // depth slots of 5 x R_total doubles
    long long *done;    // depth slots of R_total: the step whose frame the slot holds, per replica
    long long n_total;  // particles of the handle (unpadded)
    long long pk_base;  // the group's first value in the handle's packed arrays
    int R_total, rep_base, every, depth;
};

// Device pointers of one handle (all replicas packed; see tis_engine.cu).
struct Dev {
    int R, P, nblk, C;          // replicas, padded particles, particle blocks, cells
    int fp64;                   // 1: FP64 mode
    int noise;                  // tis_noise
    const RepParams *rp;
    RepState *rs;
    const int *blk_rep;         // replica of every particle block
    const int *rep_of;          // replica of every particle (padded slots included)
    double *x, *y, *z, *xo, *yo, *zo, *vx, *vy, *vz;
    int4 *q;                    // fixed-point position + (type | kind << 8 | active << 16)
    unsigned long long *f, *flr;  // 3P each: int64 fixed point (mixed) or double (FP64)
    double *gnoise;             // R x kNoise
    // cells
    int *cell_of, *cell_count, *cell_start, *cell_fill, *cell_list;
    int4 *qs;                   // packed positions in cell order (qs[slot] = q[cell_list[slot]])
    int full_lists;             // 1: SR list is the reference's full set; 0: pruned to possible forces
    int search_warps;           // warps of the pair-search grid
    int sm_count;               // multiprocessors (grid size of the rebuild kernels)
    int nc_max;                 // most cells of one replica
    int cell_smem;              // dynamic shared bytes of the cell kernel (0: its counters stay in global memory)
    // neighbour lists, column-major: nbr[k * P + p]
    int *nbr_sr, *n_sr, *nbr_lr, *n_lr;
    int cap_sr, cap_lr;
    // bonded partners whose LJ the reference subtracts again (reduce_forces, E:880-897),
    // column-major excl[k * P + p], k < n_excl[p] <= kExcl
    const int *excl, *n_excl;
    // topology (global particle indices)
    const int4 *bt_idx;         // a, b, c, kind
    const double2 *bt_par;      // k0, x0
    const int *st3_idx; const double *st3_nat, *st3_E; const int *st3_off;
    const int *st2_idx; const double *st2_r0, *st2_E;
    int nbt, nst3, nst2;        // bonded terms, tertiary and secondary stacks of all replicas
    const int *st2_offby_off, *st2_offby_idx;  // tertiary stacks that can switch each secondary off
    double *st_energy;          // tertiary energies of the last step (for the Contacts file)
    const int *hb_idx; const double *hb_nat, *hb_E; const int *hb_dode;
    const int *hb_aoff, *hb_aidx;   // atoms of every candidate (CSR, global ids)
    const int *hba_val, *hba_coff, *hba_cidx, *hba_n;
    const int *ca_list;             // atoms whose candidate count exceeds their valence
    const int *ca_coff, *ca_cidx;   // candidates of each such atom (CSR; replica-local bond numbers)
    const int *hb_coff, *hb_cpos;   // such atoms of each candidate (CSR; replica-local numbers in ca_list)
    int *hb_status, *hb_excess, *hb_active, *hb_K, *hb_A, *ca_exc;
    double *hb_energy;
    int *hb_code;               // imaging branch of the three native dihedrals
    double *hb_term;            // six restraint terms per candidate (global scratch)
    int *hb_br;                 // three dihedral branches per candidate (global scratch)
    int hb_nmax, ca_nmax, k_nmax;   // largest per-replica candidate, over-valence atom and K counts
    int cidx_max, cpos_max;         // largest per-replica ca_cidx and hb_cpos lengths
    int hb_smem;                // dynamic shared bytes of the H-bond kernel (0: its arrays stay in global scratch)
    double *eterm;              // R x kNE (per-term energies, compute_forces only)
    double *shift;              // R x 3, recentring shift of the current step (adjust_box)
    const int *cell_rep;        // replica of every cell
    int *hb_rec;                // when not null: 1 per H-bond candidate formed after the step's Monte Carlo, else 0
    int lanes_sr, lanes_lr;     // threads per particle of the step's SR (1, 2, 4) and LR (2, 4, 8) pair launches
    unsigned long long *fprof;  // when not null: the fused step kernel's phase times, kFusedPhases per replica (ns)
    FrameRing fr;               // frame output from inside the step (fr.every = 0: off)
};
constexpr int kFusedPhases = 12;  // forces, H-bond chain, shift, move, control, rebuild, steps with LR, rebuild steps,
                                  // and the H-bond chain's restraint terms, Monte Carlo, forces, Gaussians

// Adjoint work of one handle (tis_adjoint.cu).  Arrays of 3P or 9P values are
// component-major (c * P + p) like the state arrays.
constexpr int kNParams = 16;    // force-field parameters (TIS_N_PARAMS)
struct AdjDev {
    const double *st2_dss;      // d st_E / d ss_D of every secondary stack
    const int *st2_cls;         // its 5' base (0 A, 1 C, 2 G, 3 U; -1 none)
    const double *hb_dhs;       // d hb_E / d hs_D of every H-bond candidate
    int nhb;                    // H-bond candidates of all replicas
    double *lam;                // 9P: adjoint of (x, x_old, v)
    double *lamf, *mu, *jv;     // 3P: adjoint of the step's force; of the held LR force; J lambda
    double *cen;                // R x 3: adjoint of the recentring shift
    double *dth;                // R x kNParams: parameter gradient
    double *rx, *rf, *rg;       // recorded step: 9P state before it, 3P force, R x kNoise Gaussians
    int *rhb, *rlr;             // recorded step: H-bonds formed (per candidate), LR refreshed (per replica)
    const double *px, *py, *pz; // positions the pair and restraint terms are evaluated at
};

// Byte offsets of the H-bond kernel's shared-memory arrays (one replica's working
// set; the kernel and the engine's size check both use this layout).
struct HbLayout {
    size_t en, term, st, code, br, exc, al, kl, ca_off, ca_idx, hb_off, hb_pos, total;
};
__host__ __device__ inline HbLayout hb_layout(int hb_nmax, int ca_nmax, int k_nmax, int cidx_max, int cpos_max)
{
    HbLayout L;
    size_t o = 0;
    L.en = o; o += 8 * (size_t)hb_nmax;              // double per candidate
    L.term = o; o += 48 * (size_t)hb_nmax;           // six doubles per candidate
    L.st = o; o += 4 * (size_t)hb_nmax;
    L.code = o; o += 4 * (size_t)hb_nmax;
    L.br = o; o += 12 * (size_t)hb_nmax;             // three ints per candidate
    L.exc = o; o += 4 * (size_t)ca_nmax;
    L.al = o; o += 4 * (size_t)ca_nmax;
    L.kl = o; o += 4 * (size_t)k_nmax;
    L.ca_off = o; o += 4 * ((size_t)ca_nmax + 1);
    L.ca_idx = o; o += 4 * (size_t)cidx_max;
    L.hb_off = o; o += 4 * ((size_t)hb_nmax + 1);
    L.hb_pos = o; o += 4 * (size_t)cpos_max;
    L.total = (o + 15) / 16 * 16;
    return L;
}

// Launchers (stream-ordered; gated per replica on device flags where noted).
void launch_quantize(const Dev &d, cudaStream_t s);
// the group's state packed (replicas end to end, n values per array, nine arrays) <-> device
void launch_put_state(const Dev &d, cudaStream_t s, const double *stage, int n);
void launch_get_state(const Dev &d, cudaStream_t s, double *stage, int n, unsigned mask);
void launch_energies(const Dev &d, cudaStream_t s, double *out);  // 5 values per replica
void launch_clear_err(const Dev &d, cudaStream_t s);              // RepState::err = 0 for every replica
void launch_list_peaks(const Dev &d, cudaStream_t s, int *out);   // max n_sr, max n_lr (out zeroed first)
// per RNA bead of replica r: ions of `kind` within sqrt(r2cut) of it if it is a P (-1 otherwise);
// hit[j] set for each such ion (replica-local index)
void launch_ion_counts(const Dev &d, cudaStream_t s, int r, int nrna, int kind, double r2cut, int *count, int *hit);
// excl_in_list: the hot path skips the LJ of bonded pairs in the SR kernel and
// does not subtract it in the bonded kernel (the reference's net force, without
// the cancellation of two large equal terms); false gives the reference's
// per-term split (tis_compute_forces).
void launch_pair_sr(const Dev &d, cudaStream_t s, bool energies, bool excl_in_list);
void launch_pair_lr(const Dev &d, cudaStream_t s, bool energies, bool force_all);
void launch_topology(const Dev &d, cudaStream_t s, int mask, bool energies, bool make_noise, bool excl_in_list);
void launch_noise(const Dev &d, cudaStream_t s);  // the step's Gaussians only
int configure_kernels(const Dev &d);
              // kernel attributes (shared-memory limits); cudaError_t
void launch_integrate(const Dev &d, cudaStream_t s);  // recentring shift, then the particles
void launch_rebuild(const Dev &d, cudaStream_t s);  // gated on RepState::rebuild: cells, then pair search
// the parts of launch_integrate and launch_rebuild, for stage timing
void launch_shift(const Dev &d, cudaStream_t s);
void launch_move(const Dev &d, cudaStream_t s);
void launch_cells(const Dev &d, cudaStream_t s);
void launch_search(const Dev &d, cudaStream_t s);
void launch_force_all_rebuild(const Dev &d, cudaStream_t s);
void launch_rg(const Dev &d, cudaStream_t s, int replica, double *out);
int kernel_launches_per_step();
// the persistent fused step kernel: `steps` whole steps of every replica, a cluster
// of `ctas` CTAs (1..8) per replica; returns the launch's cudaError_t
int launch_step_fused(const Dev &d, cudaStream_t s, int steps, int ctas);
size_t fused_smem(const Dev &d);

// ion density grids (tis_density.cu): the least-squares fit of replica r's beads idx
// (replica-local) onto ref (3 per bead) into out[16] (R, frame centroid, reference
// centroid, rmsd); every particle of `kind` of replica r (n particles), moved by the
// fit when fit != null, binned into grid (dims[0] x dims[1] x dims[2], z fastest)
void launch_fit(const Dev &d, cudaStream_t s, int r, int n_fit, const int *idx, const double *ref, double *out);
void launch_density(const Dev &d, cudaStream_t s, int r, int n, int kind, const double *fit, const double lo[3],
                    double delta, const int dims[3], unsigned long long *grid);

// adjoint (tis_adjoint.cu).  mode 0: dU/dtheta into a.dth at positions a.px..;
// mode 1: a.jv += J tan and the parameter terms of lambda = tan.
void launch_adj_pair(const Dev &d, const AdjDev &a, cudaStream_t s, bool lr, const double *tan, int mode);
void launch_adj_topo(const Dev &d, const AdjDev &a, cudaStream_t s, const double *tan, int mode);
// the reverse pass of one recorded step: a.lam (after the step) -> a.lam (before it)
void launch_adj_step(const Dev &d, const AdjDev &a, cudaStream_t s);
// records the step's inputs into a.rx, a.rf, a.rlr (after the forces, before the integrator)
void launch_adj_record(const Dev &d, const AdjDev &a, cudaStream_t s);
// packed host-order state arrays (tis_set_states layout) <-> 9P device arrays
void launch_adj_unpack(const Dev &d, cudaStream_t s, double *dst, const double *stage, int n, unsigned mask);
void launch_adj_pack(const Dev &d, cudaStream_t s, const double *src, double *stage, int n);

}  // namespace tis
