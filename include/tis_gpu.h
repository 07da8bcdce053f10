/* tis_gpu.h — C ABI of the GB300 (sm_103a) TIS-RNA Langevin engine.
 *
 * The reference (naotohori/16S-central-folding, src/16SCD_Mg_Cl_K_COPY_fast.cpp,
 * cited as E:) has no library interface: its hot path is the call sequence
 *     populate_lists();                                   E:6237 (and from check_shifts)
 *     for (klok ...) { deterministic_forces_MPI();        E:6380  (E:2524-2586)
 *                      full_forces();                     E:6382  (E:2590-2625)
 *                      move_rigid_units();                E:6384  (E:2660-2732)
 *                      check_shifts(); }                  E:6386  (E:1741-1776)
 * acting on 1-based FP64 global arrays set up by read_maxi_key / read_PDB /
 * initialize_* / set_box / add_crowder (E:6111-6179).  Each entry point below
 * names the reference routine it replaces.  Plain pointers and sizes only.
 *
 * Conventions
 *   - Every function returns 0 (TIS_OK) or a positive TIS_ERR_* code; the text
 *     of the last error of the calling thread is available from tis_last_error.
 *   - Particle indices are 0-based (reference index minus one).
 *   - A handle owns device memory for n_replicas independent replicas that are
 *     advanced together; calls on one handle are serialised on its CUDA stream;
 *     a handle is not thread-safe; distinct handles may be used concurrently.
 *   - Host buffers passed in are copied; the library never retains them.
 */
#ifndef TIS_GPU_H
#define TIS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TIS_ABI_VERSION 1

enum tis_status {
    TIS_OK = 0,
    TIS_ERR_ARG = 1,        /* bad argument or missing system array */
    TIS_ERR_IO = 2,         /* input file cannot be opened or read */
    TIS_ERR_FORMAT = 3,     /* input file content not understood */
    TIS_ERR_CUDA = 4,       /* CUDA runtime error (no device, launch failure ...) */
    TIS_ERR_CAPACITY = 5,   /* a neighbour list overflowed its per-particle capacity */
    TIS_ERR_NONFINITE = 6,  /* non-finite force, position or velocity */
    TIS_ERR_RANGE = 7,      /* a particle left the range the cell grid covers */
    TIS_ERR_STATE = 8,      /* call out of order (e.g. forces before lists) */
    TIS_ERR_NOMEM = 9,      /* host or device allocation failed */
    TIS_ERR_SETUP = 10      /* ion placement did not converge */
};

/* array element types of tis_system arrays */
enum tis_dtype { TIS_F64 = 0, TIS_I32 = 1, TIS_I64 = 2 };

/* Text of the last error raised on the calling thread (empty if none). */
int tis_last_error(char *buf, size_t n);

/* ------------------------------------------------------------------------ */
/* Systems: host-side topology + initial state of one replica.               */
/* ------------------------------------------------------------------------ */
typedef struct tis_system tis_system;

typedef struct tis_load_params {
    const char *pdb;          /* coordinates (read_PDB, E:3137) */
    const char *bonds;        /* hydrogen-bond candidates (initialize_unprocessed_bonds, E:3733) */
    const char *stacks;       /* tertiary stacks (initialize_unprocessed_stacks, E:4232) */
    const char *maxikey;      /* 9-type parameter table (read_maxi_key, E:2883) */
    double T;                 /* -T, temperature in kcal/mol (E:6090) */
    double ss_D, hs_D, st_D;  /* -D -E -d force-field adjustments (E:6086-6089) */
    int32_t seed;             /* -s; seeds srand(T*1000*seed) (E:6105) and the Philox stream */
    double box;               /* cubic box side, A (E:6076: 350) */
    double rc;                /* Coulomb cutoff, A (E:348: 50) */
    double c_mg, c_k;         /* -c -f bulk concentrations, M (E:6092-6094) */
    int32_t n_mg, n_cl, n_k;  /* explicit ion numbers; all < 0 selects the rule of E:6167-6171 */
    int32_t center;           /* 1-based recentring bead (E:2670, E:4542: 500) */
    int32_t rng;              /* 0: glibc rand() for set-up draws, 1: Philox stream */
    int32_t reserved[7];
} tis_load_params;

/* Fills p with the reference's defaults (src/run_sample.sh and E:6076, E:348). */
int tis_load_params_default(tis_load_params *p);

/* Reads the four input files and runs the reference's set-up sequence
 * (read_maxi_key, read_PDB, initialize_HB_atoms, initialize_unprocessed_bonds,
 * initialize_unprocessed_stacks, set_box, add_crowder; E:6111-6179). */
int tis_system_load(const tis_load_params *p, tis_system **out);

/* An empty system to be filled array by array (names of the TISB system export). */
int tis_system_new(tis_system **out);
int tis_system_set(tis_system *s, const char *name, int dtype, const void *data, int64_t count);
/* Borrowed view of an array; valid until the array is replaced or s destroyed. */
int tis_system_get(const tis_system *s, const char *name, int *dtype, const void **data, int64_t *count);
/* Number of arrays and the name of array i (for enumeration). */
int tis_system_count(const tis_system *s, int *n);
int tis_system_name(const tis_system *s, int i, const char **name);
int tis_system_destroy(tis_system *s);

/* ------------------------------------------------------------------------ */
/* Engine                                                                    */
/* ------------------------------------------------------------------------ */
typedef struct tis_handle tis_handle;

enum tis_precision {
    TIS_PREC_MIXED = 0, /* FP32 pair/bonded math, int64 fixed-point forces, FP64 integration */
    TIS_PREC_FP64 = 1   /* FP64 throughout (the plain GPU path) */
};

enum tis_noise { TIS_NOISE_REFERENCE = 0, TIS_NOISE_OFF = 1 };

typedef struct tis_run_params {
    int32_t precision;     /* tis_precision */
    int32_t noise;         /* tis_noise: REFERENCE = 3000 shared Gaussians per step (E:2590-2625) */
    double sr;             /* SR list radius minus skin (E:6229: 12) */
    double skin;           /* Verlet skin dr1 (E:6227: 3) */
    int32_t lr_interval;   /* LR Coulomb refresh period (E:2550: 10) */
    int32_t cap_sr;        /* SR neighbours per particle (0: default) */
    int32_t cap_lr;        /* LR neighbours per particle (0: default) */
    int32_t device;        /* CUDA device ordinal */
    int32_t use_graph;     /* 1: tis_step replays a captured CUDA graph */
    int32_t graph_steps;   /* steps per captured graph (0: default) */
    int32_t full_lists;    /* 1: keep every SR pair within sr+skin (the reference's SR list, E:1626);
                              0 (default): a pair with a sugar or base bead is kept only within its
                              LJ range plus the skin, the only pairs that can exert a force before
                              the next rebuild */
    int32_t groups;        /* replica groups whose step graphs run concurrently on the GPU
                              (0: (3 n + 15) / 16 for n replicas, 12 for 64); results do not depend on it */
    int32_t lanes_sr;      /* threads per particle of the step's SR pair launch: 1, 2, 4 (0: 1) */
    int32_t lanes_lr;      /* threads per particle of the step's LR pair launch: 2, 4, 8 (0: 4); in mixed
                              precision results do not depend on either (fixed-point sums) */
    int32_t fused_ctas;    /* 0: a step is the chain of separate kernels (pair, bonded, H-bond, integrator,
                              rebuild); 1..8: tis_step runs the persistent fused step kernel, in which one
                              thread-block cluster of fused_ctas CTAs per replica runs whole steps back to
                              back (one launch per replica group and call, or per graph replay with
                              use_graph); mixed-precision results are the same bit for bit */
    int32_t reserved[1];
} tis_run_params;

int tis_run_params_default(tis_run_params *p);

/* Uploads n_replicas systems (each with its own size, ions, T and seed) and
 * allocates the device state.  Replaces the reference's globals set-up. */
int tis_create(const tis_system *const *systems, int n_replicas, const tis_run_params *p, tis_handle **out);
int tis_destroy(tis_handle *h);

/* State of one replica: positions, previous positions (x_old) and velocities,
 * FP64, length n each (the reference's x,y,z,x_old,..,vz, E:155-165). */
int tis_set_state(tis_handle *h, int replica, const double *x, const double *y, const double *z,
                  const double *xo, const double *yo, const double *zo,
                  const double *vx, const double *vy, const double *vz);
int tis_get_state(tis_handle *h, int replica, double *x, double *y, double *z,
                  double *xo, double *yo, double *zo, double *vx, double *vy, double *vz);

/* The state of every replica in one call: each array holds the replicas' particles
 * end to end (replica 0's n_0 values, then replica 1's, ...; total the sum of
 * tis_replica_size), one host-device copy per array and replica group.  Null
 * arrays are skipped by tis_get_states; tis_set_states needs all nine.  No
 * counterpart in the reference, which holds one system per process. */
int tis_set_states(tis_handle *h, const double *x, const double *y, const double *z,
                   const double *xo, const double *yo, const double *zo,
                   const double *vx, const double *vy, const double *vz);
int tis_get_states(tis_handle *h, double *x, double *y, double *z,
                   double *xo, double *yo, double *zo, double *vx, double *vy, double *vz);

/* populate_lists (E:1546-1737) for every replica: cell binning, SR/LR neighbour
 * lists, hydrogen-bond candidate status; resets PROGRESS (E:6238). */
int tis_populate_lists(tis_handle *h);

/* Cell of every particle (0-based linear index of E:1536) and the grid dims. */
int tis_get_cells(tis_handle *h, int replica, int32_t *cell, int32_t *dims);
/* Unordered pair set of list `which` (0: SR, 1: LR) as (i<j) pairs, 2 ints each;
 * *n receives the number of ints; at most cap ints are written. */
int tis_get_pairs(tis_handle *h, int replica, int which, int32_t *pairs, int64_t cap, int64_t *n);
/* Hydrogen-bond candidate status (-1/0) and HB_EXCESS after the last list build. */
int tis_get_hb_status(tis_handle *h, int replica, int32_t *status, int32_t *excess);

/* Force terms, for per-term parity on the current state of one replica.
 * term_mask bits: */
enum tis_term {
    TIS_TERM_SR = 1,      /* SR_interactions_lists  E:1783 (LJ + Coulomb inside 15 A) */
    TIS_TERM_LR = 2,      /* LR_interactions_lists  E:1851 (Coulomb 15 A .. rc+3 A) */
    TIS_TERM_BONDED = 4,  /* polymer_constraints    E:2354 (bonds, angles, LJ exclusions) */
    TIS_TERM_STACK = 8,   /* stacking_interactions  E:1911 */
    TIS_TERM_HB = 16      /* hydrogen_bonds_interactions E:2145 (consumes MC draws) */
};
/* energies[TIS_N_ENERGIES] (may be NULL) */
enum tis_energy_index {
    TIS_E_LJ = 0, TIS_E_COUL_SR, TIS_E_COUL_LR, TIS_E_BOND, TIS_E_ANGLE, TIS_E_EXCL,
    TIS_E2_STACK, TIS_E3_STACK, TIS_E2_HB, TIS_E3_HB, TIS_E_RG, TIS_N_ENERGIES
};
/* Sum of the selected terms into forces[3n] (x,y,z interleaved, FP64). */
int tis_compute_forces(tis_handle *h, int replica, int term_mask, double *forces, double *energies);

/* One reference step per call of each, in the reference's order, for every
 * replica (drop-in replacements of the four routines of the run loop). */
int tis_deterministic_forces(tis_handle *h); /* deterministic_forces_MPI  E:2524 */
int tis_full_forces(tis_handle *h);          /* full_forces               E:2590 */
int tis_move_rigid_units(tis_handle *h);     /* move_rigid_units          E:2660 (also measures the
                                                shifts of check_shifts, E:1745-1766) */
int tis_check_shifts(tis_handle *h);         /* check_shifts              E:1741 (list rebuild) */
/* The force array of one replica as it stands (after tis_deterministic_forces:
 * the reference's fx,fy,fz after the Allreduce, E:2576-2585), x,y,z interleaved. */
int tis_get_forces(tis_handle *h, int replica, double *forces);

/* n steps of the whole sequence for every replica; asynchronous: returns after
 * enqueueing.  With use_graph the steps replay CUDA graphs that hold every replica
 * group's branch (one launch for the whole handle): the graph of graph_steps
 * steps n / graph_steps times, then a graph of the remaining n % graph_steps steps,
 * kept for the next call with the same remainder; the graphs are captured on first
 * use and again after the lists grow. */
int tis_step(tis_handle *h, int64_t n);
/* Captures (again) the CUDA graph of `steps` fused steps of the whole handle,
 * building the lists first when needed, and makes `steps` the graph length;
 * later tis_step calls replay it for every whole `steps` (no counterpart in the
 * reference; tis_step captures on its first call otherwise). */
int tis_capture_graph(tis_handle *h, int32_t steps);
/* Waits for the handle's stream; reports device-side error flags. */
int tis_sync(tis_handle *h);

/* E2_HB, E3_HB, E2_STACK, E3_STACK of the last step and Rg of the RNA
 * (the five columns of the Energies file, E:6312). */
int tis_get_energies(tis_handle *h, int replica, double *out5);
/* The same five values for every replica: out[5 * replica + k]. */
int tis_get_all_energies(tis_handle *h, double *out);

/* Bound-ion counts on the device (the reference's analysis/mg_correlation/
 * mg_bound.F90:94-116 and analysis/salt_nt/dcd_traj_SaltCount_Kinetics_PBC.py:
 * 42-70, which read them back from trajectory files): for every phosphate of the
 * replica, in bead order, the number of ions of `kind` (3 Mg, 4 Cl, 5 K, the
 * reference's part_key; 0 counts the other phosphates) whose minimum-image FP64
 * distance is at most `radius` (at most the SR radius, e.g. 4.4, 5 or 7.2684 A);
 * *n_p receives the number of phosphates (at most cap counts are written) and
 * *total the number of distinct particles within range of some phosphate.  Summed
 * over frames at radius 7.3 A these give analysis/salt_nt/integrate_num_ions.py's
 * contact concentrations (count / (frames 4/3 pi r^3 6.02214e-4), mol/L). */
int tis_ion_counts(tis_handle *h, int replica, int kind, double radius, int32_t *counts, int64_t cap,
                   int64_t *n_p, int32_t *total);

/* Topology and trajectory files for analysis tools (the reference's
 * analysis/make_ninfo/16SCD_ninfo.cpp:6563-6650 writes the PSF; its analyses read
 * DCD trajectories).  tis_write_psf: the system's beads and ions with the
 * exporter's names, residue numbers, charges and masses, and the chain's P-S, S-B,
 * S-P bonds.  tis_write_dcd: appends the replica's current positions as one
 * CHARMM/NAMD DCD frame (single precision), writing the header first when the
 * file does not exist and updating its frame count; nsavc: steps per frame,
 * delta: the time step in the header. */
int tis_write_psf(const tis_system *s, const char *path);
/* The coarse-grained PDB of the same exporter (16SCD_ninfo.cpp:6479-6561): six
 * RECORD count lines, the beads (S, <base>b, P of residue R<base>), TER, the ions,
 * TER; coordinates x, y, z of n_particles each (NULL: the system's own). */
int tis_write_cgpdb(const tis_system *s, const double *x, const double *y, const double *z, const char *path);
/* The native-structure information file (CafeMol .ninfo) of the same exporter
 * (analysis/make_ninfo/16SCD_ninfo.cpp:6473-6477, its write_ninfo_bond_angle,
 * write_ninfo_basestack and write_ninfo_basepair): bond and angl records of the
 * chain, tbs-dist/angl/dihd of the tertiary stacks and bs-dist/dihd of the
 * secondary stacks, hb-dist/angl/dihd of every H-bond candidate, with the loaded
 * system's parameters and natives (the record layout the exporter writes, before
 * the hand edits of its do.sh). */
int tis_write_ninfo(const tis_system *s, const char *path);
int tis_write_dcd(tis_handle *h, int replica, const char *path, int32_t nsavc, double delta);

/* Ion density grid of one replica accumulated on the device over frames (the
 * reference's analysis/Mg_distribution_3D/calc_Mg_density.py:118-150, which bins
 * Mg positions read back from trajectory files with numpy.histogramdd, after
 * bestfit_motifs.py:51-58 superposed each frame on a reference structure by the
 * beads of a motif).  Bins of `delta` A from the lower corner lo, dims[0] x dims[1]
 * x dims[2] of them (the upper faces belong to the last bins).  With n_fit > 0
 * each frame is first superposed, by the least-squares rotation and translation
 * of beads fit_beads[] (replica-local indices) onto fit_ref[3 * i ..], and the
 * ions are moved with it.  tis_density_add bins the replica's current frame on
 * the handle's stream (no host synchronisation); tis_density_get returns the
 * counts (x slowest, z fastest), the frames added and the last fit's rmsd. */
typedef struct tis_density tis_density;
int tis_density_create(tis_handle *h, int replica, int kind, const double lo[3], double delta,
                       const int32_t dims[3], int32_t n_fit, const int32_t *fit_beads, const double *fit_ref,
                       tis_density **out);
int tis_density_add(tis_density *g);
int tis_density_get(tis_density *g, double *counts, int64_t cap, int64_t *frames, double *rmsd);
/* The grid as an OpenDX file (the format calc_Mg_density.py exports and
 * search_dx_maxvalue.py reads): six comment lines, the gridpositions object with
 * the origin at the centre of the first bin, three delta lines, the
 * gridconnections object, the data array of counts three per line, the field. */
int tis_density_write_dx(tis_density *g, const char *path);
/* Destroying the handle releases its grids' device memory: later calls on such a
 * grid return TIS_ERR_STATE; tis_density_destroy still frees the object. */
int tis_density_destroy(tis_density *g);

/* Frames written from inside the step (the reference writes its output every
 * 10^6 steps from the run loop, E:6276-6376, stopping the run to do it).  After
 * tis_frames_start, every `every` steps (step numbers, klok, that are multiples of
 * it) the step's own integrator kernel writes each replica's positions, its five
 * Energies-file values (E2_HB, E3_HB, E2_STACK, E3_STACK, Rg) and then the step
 * number into a ring of `depth` (>= 2) slots of pinned host memory that the GPU
 * writes directly; it adds no launch and no synchronisation to the run, graphs
 * included.  tis_frames_read copies the frame of step klok (positions packed as
 * tis_get_states packs them; energies 5 per replica) once every replica's part is
 * complete, waiting for the handle's stream only when the frame is not yet
 * written; TIS_ERR_STATE when the ring has overwritten it (read each frame before
 * `depth` more frames are written) or the run never wrote it.  One ring per
 * handle; tis_frames_stop (or tis_destroy) frees it. */
typedef struct tis_frame_ring tis_frame_ring;
int tis_frames_start(tis_handle *h, int32_t every, int32_t depth, tis_frame_ring **out);
int tis_frames_read(tis_frame_ring *f, int64_t klok, double *x, double *y, double *z, double *energies);
int tis_frames_stop(tis_frame_ring *f);

/* Appends one frame of a replica to the reference's three output files (any may
 * be NULL): the Contacts file ("%+.3f " per tertiary stack energy, then a
 * newline, E:6290-6294), the Coordinates file (x, y, z, each as the reference's
 * 1-based array of n+1 doubles with the unused index 0 written as 0, E:6298-6304)
 * and the Energies file ("%le %le %le %le %le\n": E2_HB, E3_HB, E2_STACK,
 * E3_STACK as the sum of the stack energies, Rg, E:6308-6312). */
int tis_write_frame(tis_handle *h, int replica, const char *contacts, const char *coordinates,
                    const char *energies);
/* The restart read of E:6181-6211: the last complete frame of a Coordinates file
 * of n particles into x, y, z (n values each, any may be NULL) and the number of
 * frames in *frames (the reference resumes at klok = frames * 10^6). */
int tis_read_last_frame(const char *coordinates, int n, double *x, double *y, double *z, int64_t *frames);
/* Energies of the tertiary stacks of the last step (the Contacts file, E:6290). */
int tis_get_stack_energies(tis_handle *h, int replica, double *out, int64_t cap, int64_t *n);
/* Step counter (klok), rebuild count and rand() draws consumed by one replica. */
int tis_get_counters(tis_handle *h, int replica, int64_t *klok, int64_t *rebuilds, int64_t *draws);

/* Bit-exact checkpoint of the whole engine state (no counterpart in the reference,
 * whose restart, tis_read_last_frame, resumes from positions only): x, x_old, v,
 * the held LR force, every replica's counters and rand() position, the neighbour
 * lists and H-bond status of every replica group.  A handle created with the same
 * systems and run parameters continues from a loaded checkpoint exactly as the
 * saving handle would have continued (bit for bit in mixed precision).  The file
 * records a hash of the replicas' sizes, parameters and seeds; tis_checkpoint_load
 * reads and checks the whole file (format, groups, sizes, that hash) before it
 * changes anything, and on TIS_ERR_FORMAT / TIS_ERR_IO leaves the handle as it was. */
int tis_checkpoint_save(tis_handle *h, const char *path);
int tis_checkpoint_load(tis_handle *h, const char *path);

/* Number of replicas, particles of one replica, and the CUDA stream (cudaStream_t). */
int tis_get_info(tis_handle *h, int *n_replicas, int *device, void **stream);
int tis_replica_size(tis_handle *h, int replica, int *n_particles);

/* Runs n steps with direct launches, one kernel after another, and CUDA events
 * between them, on each group's stream; ms[TIS_N_STAGES] receives the mean
 * duration per step, summed over the replica groups, of: SR pair forces, LR pair
 * forces, bonded + stacking terms, H-bonds + the step's Gaussians, recentring
 * shift, integrator (+ skin check), cell binning, pair search. */
#define TIS_N_STAGES 8
int tis_profile_stages(tis_handle *h, int64_t n, double *ms);

/* The same eight kernels timed inside the step as it runs (no counterpart in the
 * reference): `steps` (1..1000) fused steps of every group captured with CUDA
 * events around each kernel, all groups' graphs replayed concurrently;
 * ms[TIS_N_STAGES] receives each kernel's mean duration per launch (one group,
 * one step), averaged over the steps and groups, with the other groups' work
 * running beside it.  Advances every replica by `steps` steps. */
int tis_profile_in_step(tis_handle *h, int32_t steps, double *ms);

/* The persistent fused step kernel (tis_run_params.fused_ctas) run for `steps`
 * steps of every replica, with `ctas` CTAs per replica and its phase timer on (no
 * counterpart in the reference): out[0..5] = mean microseconds per step of the
 * force phase, of the H-bond chain inside it (terms, Monte Carlo, Gaussians),
 * the recentring shift, the integration, the control step, and the list rebuild
 * per step that rebuilds; out[6] = share of steps that refresh the LR force,
 * out[7] = list rebuilds per step; out[8..11] = microseconds per step of the
 * H-bond chain's restraint terms, Monte Carlo, forces and Gaussians (out has 12
 * values); means over the replicas.  Advances every replica by `steps` steps. */
int tis_profile_fused(tis_handle *h, int32_t steps, int32_t ctas, double *out);

/* Kernel launches enqueued by tis_step since the handle was created. */
int tis_get_launch_count(tis_handle *h, int64_t *n);

/* Draws first .. first+n-1 of the rand() stream that replaces glibc rand() for
 * a replica with this seed: Philox-4x32-10 (Salmon et al. 2011), values in
 * [1, 2^31-1].  The hydrogen-bond Monte Carlo (E:2251-2300) and full_forces
 * (E:2594-2606) consume it in the reference's order. */
int tis_rand_stream(uint64_t seed, uint64_t first, int64_t n, int32_t *out);

/* Measured choice of the launch configuration (no counterpart in the reference):
 * replica groups, steps per captured graph, the threads per particle of the SR
 * and LR pair launches and the step path (fused_ctas: the separate kernels, or
 * the persistent fused kernel with 1, 2 or 4 CTAs per replica), tuned one after
 * another (coordinate descent), for calls of `steps` steps (0: 300): each trial
 * times, with CUDA events on the handle's stream, as many tis_step(steps) calls of
 * the given replicas as make up at least 1000 steps, after a warm-up that captures
 * the graphs they replay.  *best receives base with the chosen values and *rate (if
 * not NULL) the measured replica-steps/s.  When `cache` names a file, a line for
 * the same workload (replicas, particles, box, cutoff, precision, steps per call,
 * device) is reused without trials, and a new result is appended. */
int tis_autotune(const tis_system *const *systems, int n_replicas, const tis_run_params *base, int64_t steps,
                 const char *cache, tis_run_params *best, double *rate);

/* ------------------------------------------------------------------------ */
/* Parameter derivatives (no counterpart in the reference)                    */
/* ------------------------------------------------------------------------ */
/* The force-field parameters theta, in this order, as the reference defines them:
 *   0-3  ss_D of the secondary stacks whose 5' base is A, C, G, U (the -D flag,
 *        split by 5' base; st_E = e0 + ss_D / c + s (T - T0), E:4397-4427)
 *   4    st_D, tertiary stacking strength (-d; st_E = -st_D, E:4344)
 *   5    hs_D, H-bond strength (-E; hb_E = -0.73753 hs_D per bond of a candidate,
 *        E:3881, E:3963)
 *   6-11 ELJ of P, S, the four bases (one pooled value), Mg, Cl, K (MAXIKEY;
 *        E_LJ = sqrt(ELJ_i ELJ_j), E:2930)
 *   12-13 RLJ of Mg and K (the contact distance R_i + R_j of pairs with an ion,
 *        E:2918-2922, and the friction 0.555 RLJ of the ion, E:2897-2903)
 *   14   lB, the Coulomb strength 332.06 (0.0327 T - 0.0067) (E:6109)
 *   15   the Debye length lambda_D of the screened Coulomb term
 *        q_i q_j lB exp(-r / lambda_D) / r (system scalar "debye"; 0 or infinity:
 *        unscreened, the reference's truncated Coulomb E:825-855, where the
 *        derivative is 0)
 * Derivatives follow the forces: the LJ energy is the shifted WCA form
 * E_LJ (s^12 - 2 s^6 + 1) without the reporting clamp below D2_LJ_MINIMUM, bonded
 * pairs carry the net LJ weight of the force path, and discrete events (H-bond
 * Monte Carlo choices, stack switching, list membership, velocity cap, ion wrap)
 * are held as the forward pass took them. */
#define TIS_N_PARAMS 16

/* dU/dtheta of every replica at its current state: out[TIS_N_PARAMS * replica + j],
 * U the total potential (pairs, bonded, stacks, H-bonds).  The H-bond term uses
 * the bonds that the valence-limited Monte Carlo (E:2239-2315) leaves formed at
 * this state, run as a force evaluation runs it (it consumes rand() draws).  Lists
 * are rebuilt first when the state was set since the last build. */
int tis_param_grad(tis_handle *h, double *out);

/* Gradient of a loss of the final state through `steps` steps of the fused
 * Langevin step (fixed noise: the rand() stream is part of the state), starting
 * with a list build (populate_lists, as the reference's run starts).  The forward
 * pass keeps a checkpoint of the whole engine state every `checkpoint_every`
 * steps; the backward pass recomputes each interval from its checkpoint and runs
 * the adjoint of every step (integrator, recentring, the forces' Jacobian as a
 * directional derivative, the multiple-time-step LR force held between its
 * refreshes) in FP64.  seed[9]: dL/d(x, y, z, xo, yo, zo, vx, vy, vz) of the final
 * state, packed as tis_set_states packs states (any may be NULL: zero).  Output:
 * dtheta[TIS_N_PARAMS * replica + j] = dL/dtheta_j and, if dstate0 is not NULL,
 * dL/d(initial state) packed the same way (NULL entries skipped).  On return the
 * engine holds the final state of the forward pass. */
int tis_traj_grad(tis_handle *h, int64_t steps, int32_t checkpoint_every, const double *const *seed,
                  double *dtheta, double *const *dstate0);

/* ------------------------------------------------------------------------ */
/* Allocation-free list build                                                 */
/* ------------------------------------------------------------------------ */
/* No counterpart in the reference: an addition for callers that cannot allocate
 * device memory where they need a neighbour list - a host recording its CUDA work
 * into a graph (cudaMalloc cannot be captured), a time step that must not
 * synchronise the device (cudaFree does), or an engine running under a fixed,
 * pre-reserved memory budget.  It bins one configuration into cells and returns
 * the SR and LR pair sets with populate_lists' rule (E:1461-1694): SR when
 * r^2 <= sr_radius^2, otherwise LR when r^2 <= lr_radius^2 and neither bead is a
 * sugar or a base (kind 1 or 2); cells of side >= lr_radius; minimum image.
 * All pointers d_* are device memory owned by the caller: positions (FP64, n
 * each), kinds (n), pair outputs (2 ints per pair, i < j, unordered, at most
 * *_cap pairs written) and d_counts[3] = {SR pairs, LR pairs, particles outside
 * the grid's single periodic wrap}, all written on `stream` (cudaStream_t; NULL
 * = default stream); counts above the capacities mean the outputs were cut.
 * Allocates nothing: its scratch is a fixed device array of 896 KiB that every
 * GPU loading the library keeps until exit, which limits a call to 65,536
 * particles and 32,768 cells (larger calls fail with TIS_ERR_ARG).  Every call
 * reuses that one array, so calls that overlap on the GPU race: order them.  The
 * first call on a device looks up the array's address; make it before any stream
 * capture starts. */
int tis_pair_lists_noalloc(const double *d_x, const double *d_y, const double *d_z, const int32_t *d_kind,
                           int32_t n, const double *box, double sr_radius, double lr_radius,
                           int32_t *d_sr_pairs, int64_t sr_cap, int32_t *d_lr_pairs, int64_t lr_cap,
                           uint64_t *d_counts, void *stream);

#ifdef __cplusplus
}
#endif
#endif
