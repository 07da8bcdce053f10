// Engine handle: packs replicas into device arrays and implements the C ABI
// entry points of include/tis_gpu.h that drive the kernels.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "tis_host.h"
#include <nvtx3/nvToolsExt.h>

#include "tis_kernels.cuh"

using tis::fail;

#define TIS_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(TIS_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                                \
    } while (0)

namespace {

struct RepHost {
    int n, nrna, npad, p0, c0, nc, mc[3];
    int bt0, bt1, s30, s31, s20, s21, hb0, hb1, hba0, hba1;
};

template <class T>
int dalloc(std::vector<void *> &owned, T **p, size_t count)
{
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) return fail(TIS_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
    owned.push_back((void *)*p);
    e = cudaMemset(*p, 0, count * sizeof(T));
    if (e != cudaSuccess) return fail(TIS_ERR_CUDA, "cudaMemset: %s", cudaGetErrorString(e));
    return TIS_OK;
}

template <class T>
int dupload(std::vector<void *> &owned, T **p, const std::vector<T> &h)
{
    int rc = dalloc(owned, p, h.size());
    if (rc) return rc;
    if (!h.empty()) {
        cudaError_t e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(TIS_ERR_CUDA, "cudaMemcpy H2D: %s", cudaGetErrorString(e));
    }
    return TIS_OK;
}

const tis::Array *need(const tis_system *s, const char *name, int r, int dtype, int64_t count = -1)
{
    const tis::Array *a = s->get(name);
    if (!a) {
        fail(TIS_ERR_ARG, "replica %d: system array '%s' missing", r, name);
        return nullptr;
    }
    if (a->dtype != dtype) {
        fail(TIS_ERR_ARG, "replica %d: system array '%s' has dtype %d, expected %d", r, name, a->dtype, dtype);
        return nullptr;
    }
    if (count >= 0 && a->count() != count) {
        fail(TIS_ERR_ARG, "replica %d: system array '%s' has %lld entries, expected %lld", r, name,
             (long long)a->count(), (long long)count);
        return nullptr;
    }
    return a;
}

double scalar_f64(const tis_system *s, const char *name, double def)
{
    const tis::Array *a = s->get(name);
    if (!a || a->count() < 1) return def;
    if (a->dtype == TIS_F64) return a->as<double>()[0];
    if (a->dtype == TIS_I64) return (double)a->as<int64_t>()[0];
    return (double)a->as<int32_t>()[0];
}

int64_t scalar_i64(const tis_system *s, const char *name, int64_t def)
{
    const tis::Array *a = s->get(name);
    if (!a || a->count() < 1) return def;
    if (a->dtype == TIS_I64) return a->as<int64_t>()[0];
    if (a->dtype == TIS_I32) return a->as<int32_t>()[0];
    return (int64_t)a->as<double>()[0];
}

int round_up(int v, int m) { return (v + m - 1) / m * m; }

// an NVTX range around one API call (header-only NVTX; no cost without a profiler)
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};

}  // namespace

// One group of replicas: its own device state, streams and CUDA graph.  A handle
// holds several groups whose step graphs run concurrently.
struct Group {
    int R = 0, P = 0, C = 0, nblk = 0;
    tis_run_params prm{};
    cudaStream_t stream = nullptr;
    cudaStream_t side[3] = {nullptr, nullptr, nullptr};  // concurrent force branches
    cudaEvent_t fork = nullptr, join[3] = {nullptr, nullptr, nullptr};
    std::vector<void *> owned;
    std::vector<RepHost> rep;
    tis::Dev dev{};
    bool lists_built = false;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    cudaGraphExec_t tail = nullptr;  // the last remainder length (n % graph_steps) captured as its own graph
    int tail_steps = 0;
    cudaEvent_t *pev = nullptr;      // when set (tis_profile_in_step): events recorded around every kernel
    int pev_next = 0;
    long long list_gen = 0;          // advanced whenever the lists move (graphs holding their pointers go stale)
    int base = 0;  // handle-wide index of the group's first replica
    long long launches = 0;
    double *d_scalar = nullptr;
    int npk = 0;              // particles of the group's replicas (unpadded)
    double *stage = nullptr;  // nine packed arrays of npk values (tis_traj_grad's seeds and state adjoints)
    double *d_e5 = nullptr;   // five energies per replica (tis_get_all_energies)
    tis::RepState *h_rs = nullptr;  // pinned host copy of the replicas' state (list build checks)
    int *h_peaks = nullptr;         // pinned: largest SR and LR neighbour counts of the last list build
    int *d_peaks = nullptr;
    // parameter-derivative coefficients (tis_param_grad, tis_traj_grad)
    double *a_st2_dss = nullptr, *a_hb_dhs = nullptr;
    int *a_st2_cls = nullptr;
    int nhb_all = 0, nhba_all = 0;  // H-bond candidates and H-bond atoms of all replicas

    ~Group()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (tail) cudaGraphExecDestroy(tail);
        for (void *p : owned) cudaFree(p);
        if (h_rs) cudaFreeHost(h_rs);
        if (h_peaks) cudaFreeHost(h_peaks);
        for (int k = 0; k < 3; ++k) {
            if (side[k]) cudaStreamDestroy(side[k]);
            if (join[k]) cudaEventDestroy(join[k]);
        }
        if (fork) cudaEventDestroy(fork);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int check_flags(Group *h)
{
    std::vector<tis::RepState> rs(h->R);
    TIS_CUDA(cudaMemcpyAsync(rs.data(), h->dev.rs, sizeof(tis::RepState) * h->R, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    for (int r = 0; r < h->R; ++r) {
        const int e = rs[r].err;
        if (e & tis::kErrCapacity) return fail(TIS_ERR_CAPACITY, "replica %d: neighbour list capacity exceeded", h->base + r);
        if (e & tis::kErrRange) return fail(TIS_ERR_RANGE, "replica %d: a particle left the cell grid's range", h->base + r);
        if (e & tis::kErrNonFinite) return fail(TIS_ERR_NONFINITE, "replica %d: non-finite or runaway force/state", h->base + r);
    }
    return TIS_OK;
}

int clear_flags(Group *h)
{
    // err is the 4th int after 4 eight-byte counters and a double; clear via a host round trip
    std::vector<tis::RepState> rs(h->R);
    TIS_CUDA(cudaMemcpyAsync(rs.data(), h->dev.rs, sizeof(tis::RepState) * h->R, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    for (auto &s : rs) s.err = 0;
    TIS_CUDA(cudaMemcpyAsync(h->dev.rs, rs.data(), sizeof(tis::RepState) * h->R, cudaMemcpyHostToDevice, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return TIS_OK;
}

void enqueue_step(Group *h);

// the captured step graphs hold the list pointers: dropped when the lists move
void drop_graphs(Group *h)
{
    ++h->list_gen;
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->tail) cudaGraphExecDestroy(h->tail);
    h->graph = h->tail = nullptr;
    h->graph_steps = h->tail_steps = 0;
}

// `steps` fused steps of the group captured from its stream into *out
int capture_steps(Group *h, int steps, cudaGraphExec_t *out)
{
    cudaGraph_t g;
    TIS_CUDA(cudaStreamSynchronize(h->stream));  // no graph of the group in flight during capture and upload
    TIS_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < steps; ++s) enqueue_step(h);
    TIS_CUDA(cudaStreamEndCapture(h->stream, &g));
    const cudaError_t e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(TIS_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    return TIS_OK;
}

int grow_lists(Group *h, int cap_sr, int cap_lr)
{
    // lists are the last allocations that depend on capacity; allocate anew
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    auto drop = [&](void *p) {
        auto it = std::find(h->owned.begin(), h->owned.end(), p);
        if (it != h->owned.end()) {
            cudaFree(p);
            h->owned.erase(it);
        }
    };
    drop(h->dev.nbr_sr);
    drop(h->dev.nbr_lr);
    int rc;
    if ((rc = dalloc(h->owned, &h->dev.nbr_sr, (size_t)cap_sr * h->P))) return rc;
    if ((rc = dalloc(h->owned, &h->dev.nbr_lr, (size_t)cap_lr * h->P))) return rc;
    TIS_CUDA(cudaDeviceSynchronize());  // the memsets (legacy stream) land before the next build
    h->dev.cap_sr = cap_sr;
    h->dev.cap_lr = cap_lr;
    drop_graphs(h);
    return TIS_OK;
}

int uncount_rebuilds(Group *h, int n)
{
    std::vector<tis::RepState> rs(h->R);
    TIS_CUDA(cudaMemcpyAsync(rs.data(), h->dev.rs, sizeof(tis::RepState) * h->R, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    for (auto &s : rs) s.rebuilds -= n;
    TIS_CUDA(cudaMemcpyAsync(h->dev.rs, rs.data(), sizeof(tis::RepState) * h->R, cudaMemcpyHostToDevice, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return TIS_OK;
}

// populate_lists for the group, in two halves around a stream synchronisation so
// that several groups' builds can run at once: the launch (flags cleared, every
// replica rebuilt, the largest neighbour counts reduced, flags and counts copied to
// pinned host memory) and the check.  The lists grow until they hold twice the
// largest neighbour count found, so that later rebuilds (ions gathering at the
// RNA, the chain compacting) have room; a step that still overflows reports
// TIS_ERR_CAPACITY.
int populate_launch(Group *h)
{
    tis::launch_clear_err(h->dev, h->stream);
    tis::launch_force_all_rebuild(h->dev, h->stream);
    // every replica rebuilds: the search gets six blocks of four warps per SM instead
    // of the step's one (a warp per particle is latency-bound; more warps in flight)
    tis::Dev full = h->dev;
    full.search_warps = h->dev.sm_count * 24;
    tis::launch_rebuild(full, h->stream);
    TIS_CUDA(cudaMemsetAsync(h->d_peaks, 0, 2 * sizeof(int), h->stream));
    tis::launch_list_peaks(h->dev, h->stream, h->d_peaks);
    TIS_CUDA(cudaGetLastError());
    TIS_CUDA(cudaMemcpyAsync(h->h_rs, h->dev.rs, sizeof(tis::RepState) * h->R, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaMemcpyAsync(h->h_peaks, h->d_peaks, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    return TIS_OK;
}

// after the group's stream is synchronised: *again when the lists must grow and be
// built once more
int populate_check(Group *h, int attempt, bool *again)
{
    *again = false;
    bool overflow = false;
    for (int r = 0; r < h->R; ++r) {
        const int e = h->h_rs[r].err;
        if (e & tis::kErrRange) return fail(TIS_ERR_RANGE, "replica %d: a particle left the cell grid's range", h->base + r);
        if (e & tis::kErrNonFinite) return fail(TIS_ERR_NONFINITE, "replica %d: non-finite or runaway force/state", h->base + r);
        overflow = overflow || (e & tis::kErrCapacity);
    }
    const int want_sr = std::max(h->dev.cap_sr, round_up(2 * h->h_peaks[0], 32));
    const int want_lr = std::max(h->dev.cap_lr, round_up(2 * h->h_peaks[1], 32));
    if (!overflow && want_sr == h->dev.cap_sr && want_lr == h->dev.cap_lr) {
        h->lists_built = true;
        // the builds discarded for capacity do not count as list rebuilds
        return attempt ? uncount_rebuilds(h, attempt) : TIS_OK;
    }
    if (attempt >= 7) return fail(TIS_ERR_CAPACITY, "neighbour lists keep overflowing");
    // an overflowing list reports its capacity as its count: grow by half at least
    const int rc = grow_lists(h, overflow ? std::max(want_sr, round_up(h->dev.cap_sr * 3 / 2, 32)) : want_sr,
                              overflow ? std::max(want_lr, round_up(h->dev.cap_lr * 3 / 2, 32)) : want_lr);
    if (rc) return rc;
    *again = true;
    return TIS_OK;
}

int populate(Group *h)
{
    for (int attempt = 0;; ++attempt) {
        int rc = populate_launch(h);
        if (rc) return rc;
        TIS_CUDA(cudaStreamSynchronize(h->stream));
        bool again = false;
        if ((rc = populate_check(h, attempt, &again)) || !again) return rc;
    }
}

// deterministic_forces_MPI (E:2524-2586): the four force kernels are independent
// (fixed-point atomics into one sum, the LR sum kept apart), so they run as
// concurrent branches joined before the integrator
// in-step profiling (tis_profile_in_step): an event recorded on s before stage k of
// the step being captured (begin) or after it; no-op otherwise.  Event pair k of a
// step sits at pev[2 * (step * TIS_N_STAGES + k)].
void mark(Group *h, cudaStream_t s, int k, bool begin)
{
    if (!h->pev) return;
    // External: captured as an event-record node of the graph (a plain record during
    // capture only orders the streams)
    cudaEventRecordWithFlags(h->pev[2 * (h->pev_next * TIS_N_STAGES + k) + (begin ? 0 : 1)], s,
                             cudaEventRecordExternal);
}

void enqueue_forces(Group *h, bool make_noise)
{
    cudaEventRecord(h->fork, h->stream);
    for (int k = 0; k < 3; ++k) cudaStreamWaitEvent(h->side[k], h->fork, 0);
    mark(h, h->side[0], 1, true);
    tis::launch_pair_lr(h->dev, h->side[0], false, false);
    mark(h, h->side[0], 1, false);
    mark(h, h->side[1], 2, true);
    tis::launch_topology(h->dev, h->side[1], 4 | 8, false, false, true);
    mark(h, h->side[1], 2, false);
    mark(h, h->side[2], 3, true);
    tis::launch_topology(h->dev, h->side[2], 16, false, make_noise, true);
    mark(h, h->side[2], 3, false);
    mark(h, h->stream, 0, true);
    tis::launch_pair_sr(h->dev, h->stream, false, true);
    mark(h, h->stream, 0, false);
    for (int k = 0; k < 3; ++k) {
        cudaEventRecord(h->join[k], h->side[k]);
        cudaStreamWaitEvent(h->stream, h->join[k], 0);
    }
}

void enqueue_step(Group *h)
{
    enqueue_forces(h, true);                   // the H-bond kernel also draws full_forces' Gaussians
    if (!h->pev) {
        tis::launch_integrate(h->dev, h->stream);  // recentring shift; last block per replica: skin check
        tis::launch_rebuild(h->dev, h->stream);
        return;
    }
    // the same four launches with events between them (their programmatic
    // dependent launch then waits for the event nodes like a plain dependency)
    void (*chain[4])(const tis::Dev &, cudaStream_t) = {tis::launch_shift, tis::launch_move, tis::launch_cells,
                                                         tis::launch_search};
    for (int k = 0; k < 4; ++k) {
        mark(h, h->stream, 4 + k, true);
        chain[k](h->dev, h->stream);
        mark(h, h->stream, 4 + k, false);
    }
    ++h->pev_next;
}

int valid_replica(Group *h, int r)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    if (r < 0 || r >= h->R) return fail(TIS_ERR_ARG, "replica %d out of range (0..%d)", r, h->R - 1);
    return TIS_OK;
}

}  // namespace


static int grp_create(const tis_system *const *systems, int n_replicas, const tis_run_params &prm, int base, Group **out)
{
    Group *h = new Group();
    h->prm = prm;
    h->R = n_replicas;
    h->base = base;
    auto bail = [&](int rc) {
        delete h;
        return rc;
    };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(TIS_ERR_CUDA, "cudaStreamCreate failed"));
    for (int k = 0; k < 3; ++k)
        if (cudaStreamCreateWithFlags(&h->side[k], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->join[k], cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(TIS_ERR_CUDA, "cudaStreamCreate/cudaEventCreate failed"));
    if (cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(TIS_ERR_CUDA, "cudaEventCreate failed"));

    std::vector<tis::RepParams> rp(n_replicas);
    std::vector<int> code, blk_rep, rep_of, cell_rep;
    std::vector<double> st[9];
    std::vector<int4> bt_idx;
    std::vector<double2> bt_par;
    std::vector<int> st3_idx, st3_off, st2_idx, hb_idx, hb_dode, hb_aoff{0}, hb_aidx, hba_val, hba_coff{0}, hba_cidx,
        hba_n, ca_list;
    std::vector<double> st3_nat, st3_E, st2_r0, st2_E, hb_nat, hb_E;
    std::vector<double> st2_dss, hb_dhs;  // parameter derivatives of st2_E (by ss_D) and hb_E (by hs_D)
    std::vector<int> st2_cls;             // 5' base of each secondary stack (0-3 A C G U; -1 unknown)
    std::vector<std::vector<int>> excl_of;
    int p0 = 0, c0 = 0, kscr = 0;
    double max_rho = 0, max_rho_ch = 0;
    const char *snames[9] = {"x", "y", "z", "ox", "oy", "oz", "vx", "vy", "vz"};

    for (int r = 0; r < n_replicas; ++r) {
        const tis_system *s = systems[r];
        if (!s) return bail(fail(TIS_ERR_ARG, "replica %d: null system", base + r));
        const int n = (int)scalar_i64(s, "n_particles", -1);
        const int nrna = (int)scalar_i64(s, "n_rna", -1);
        if (n <= 0 || nrna <= 0 || nrna > n) return bail(fail(TIS_ERR_ARG, "replica %d: bad n_particles/n_rna", base + r));
        const tis::Array *box = need(s, "box", base + r, TIS_F64, 3);
        const tis::Array *type = need(s, "type", base + r, TIS_I32, n), *kind = need(s, "kind", base + r, TIS_I32, n);
        const tis::Array *mass = need(s, "mass", base + r, TIS_F64, 9), *rlj = need(s, "rlj", base + r, TIS_F64, 9);
        const tis::Array *elj = need(s, "elj", base + r, TIS_F64, 9), *qc = need(s, "qc", base + r, TIS_F64, 9);
        if (!box || !type || !kind || !mass || !rlj || !elj || !qc) return bail(TIS_ERR_ARG);
        const tis::Array *sv[9];
        for (int k = 0; k < 9; ++k)
            if (!(sv[k] = need(s, snames[k], base + r, TIS_F64, n))) return bail(TIS_ERR_ARG);
        excl_of.resize((size_t)p0 + round_up(n, tis::kBlock));
        const int center = (int)scalar_i64(s, "center", 499);
        if (center < 0 || center >= nrna) return bail(fail(TIS_ERR_ARG, "replica %d: centre bead %d outside the RNA", base + r, center));

        RepHost hr{};
        hr.n = n;
        hr.nrna = nrna;
        hr.npad = round_up(n, tis::kBlock);
        hr.p0 = p0;
        tis::RepParams &R = rp[r];
        memset(&R, 0, sizeof R);
        const double T = scalar_f64(s, "T", 0.615), hstep = scalar_f64(s, "h", 0.05);
        const double lB = scalar_f64(s, "lB", 332.0637090 * (0.03273600947 * T - 0.00669625750));
        const double rc = scalar_f64(s, "rc", 50.0);
        // Debye length of the screened Coulomb term q_i q_j lB exp(-r / debye) / r (no
        // counterpart in the reference, whose truncated Coulomb E:825-855 is debye = 0
        // or infinity: unscreened)
        const double debye = scalar_f64(s, "debye", 0.0);
        if (rc < prm.sr) return bail(fail(TIS_ERR_ARG, "replica %d: Coulomb cutoff %g below the SR radius %g", base + r, rc, prm.sr));
        for (int k = 0; k < 3; ++k) {
            const double L = box->as<double>()[k];
            R.box[k] = L;
            R.hbox[k] = 0.5 * L;
            R.qinv[k] = 4294967296.0 / L;
            R.qstep[k] = (float)(L / 4294967296.0);
            R.mc[k] = (int)(L / (rc + prm.skin));  // E:1484-1490
            if (R.mc[k] < 1) return bail(fail(TIS_ERR_ARG, "replica %d: box smaller than the LR list radius", base + r));
            R.lcell[k] = L / R.mc[k];
            hr.mc[k] = R.mc[k];
        }
        hr.c0 = c0;
        hr.nc = R.mc[0] * R.mc[1] * R.mc[2];
        R.c0 = c0;
        R.nc = hr.nc;
        R.p0 = p0;
        R.n = n;
        R.npad = hr.npad;
        R.center = p0 + center;
        R.nrna = nrna;
        R.lr_interval = prm.lr_interval;
        R.T = T;
        R.h = hstep;
        R.lB = lB;
        R.kappa = (debye > 0.0 && std::isfinite(debye)) ? 1.0 / debye : 0.0;
        R.kappaf = (float)R.kappa;
        R.rc2 = rc * rc;
        R.r2sr = (prm.sr + prm.skin) * (prm.sr + prm.skin);
        R.r2lr = (rc + prm.skin) * (rc + prm.skin);
        R.skin = prm.skin;
        R.rc2f = (float)R.rc2;
        R.r2srf = (float)R.r2sr;
        R.r2lrf = (float)R.r2lr;
        R.Tf = (float)T;
        // read_maxi_key (E:2883-2945)
        for (int t = 1; t <= 9; ++t) {
            const double m = mass->as<double>()[t - 1], Rl = rlj->as<double>()[t - 1];
            const double visc = 0.555 * Rl;
            R.mass[t] = m;
            R.k1[t] = exp(-visc / m * hstep);
            R.k2[t] = (1.0 - R.k1[t]) / visc;
            R.sigma[t] = sqrt(2.0 * visc * T / hstep);
            R.vcap[t] = m / (300.0 * T);
            R.k2fix[t] = R.k2[t] / tis::kFixScale;
            R.k2sig[t] = R.k2[t] * R.sigma[t];
        }
        for (int a = 1; a <= 9; ++a)
            for (int b = a; b <= 9; ++b) {
                const int J = (a - 1) * 9 - (a - 1) * a / 2 + b;
                const double Dl = (a <= 6 && b <= 6) ? 3.2 : rlj->as<double>()[a - 1] + rlj->as<double>()[b - 1];
                const double El = sqrt(elj->as<double>()[a - 1] * elj->as<double>()[b - 1]);
                const double Fl = 12.0 * El / (tis::kSig0 * tis::kSig0);
                const double Q = qc->as<double>()[a - 1] * qc->as<double>()[b - 1];
                const double dmin = (Dl - 0.4406141861 * tis::kSig0) * (Dl - 0.4406141861 * tis::kSig0);
                R.dlj2_d[J] = Dl * Dl;
                R.dlj_d[J] = Dl;
                R.flj_d[J] = Fl;
                R.elj_d[J] = El;
                R.d2min_d[J] = dmin;
                R.qclb_d[J] = Q * lB;
                R.dlj2[J] = (float)(Dl * Dl);
                R.dm[J] = (float)(Dl - tis::kSig0);
                R.flj[J] = (float)Fl;
                R.elj[J] = (float)El;
                R.d2min[J] = (float)dmin;
                R.qclb[J] = (float)(Q * lB);
                R.ljkeep2[J] = (float)((Dl + prm.skin) * (Dl + prm.skin) * (1.0 + 1e-5));
            }
        R.seed = (unsigned long long)scalar_i64(s, "seed", base + r + 1);

        // particles
        for (int i = 0; i < hr.npad; ++i) {
            if (i < n) {
                const int t = type->as<int32_t>()[i], k = kind->as<int32_t>()[i];
                if (t < 1 || t > 9 || k < 0 || k > 5) return bail(fail(TIS_ERR_ARG, "replica %d: bad type/kind of particle %d", base + r, i));
                if ((i < nrna) != (k <= 2)) return bail(fail(TIS_ERR_ARG, "replica %d: RNA beads must precede the ions", base + r));
                code.push_back(t | (k << 8) | (1 << 16));
                for (int c = 0; c < 9; ++c) st[c].push_back(sv[c]->as<double>()[i]);
            } else {
                code.push_back(1);
                for (int c = 0; c < 9; ++c) st[c].push_back(0.0);
            }
            rep_of.push_back(r);
        }
        for (int b = 0; b < hr.npad / tis::kBlock; ++b) blk_rep.push_back(r);
        for (int c = 0; c < hr.nc; ++c) cell_rep.push_back(r);
        double vol = R.box[0] * R.box[1] * R.box[2];
        int nch = 0;
        for (int i = 0; i < n; ++i) nch += (kind->as<int32_t>()[i] != 1 && kind->as<int32_t>()[i] != 2);
        max_rho = std::max(max_rho, n / vol);
        max_rho_ch = std::max(max_rho_ch, nch / vol);

        // bonded terms (polymer_constraints order)
        const tis::Array *btk = need(s, "bt_kind", base + r, TIS_I32);
        if (!btk) return bail(TIS_ERR_ARG);
        const int64_t nbt = btk->count();
        const tis::Array *bta = need(s, "bt_a", base + r, TIS_I32, nbt), *btb = need(s, "bt_b", base + r, TIS_I32, nbt);
        const tis::Array *btc = need(s, "bt_c", base + r, TIS_I32, nbt), *btk0 = need(s, "bt_k0", base + r, TIS_F64, nbt);
        const tis::Array *btx0 = need(s, "bt_x0", base + r, TIS_F64, nbt);
        if (!bta || !btb || !btc || !btk0 || !btx0) return bail(TIS_ERR_ARG);
        hr.bt0 = (int)bt_idx.size();
        // the bonds first, then the angles (each in polymer_constraints order), so that
        // the threads of a warp run the same term; the force sums do not depend on it
        for (int pass = 0; pass < 2; ++pass)
            for (int64_t t = 0; t < nbt; ++t) {
                const int kd = btk->as<int32_t>()[t];
                if ((kd == 1) != (pass == 1)) continue;
                const int a = bta->as<int32_t>()[t], b = btb->as<int32_t>()[t], c = btc->as<int32_t>()[t];
                if (a < 0 || a >= nrna || b < 0 || b >= nrna || (kd == 1 && (c < 0 || c >= nrna)))
                    return bail(fail(TIS_ERR_ARG, "replica %d: bonded term %lld has a bad index", base + r, (long long)t));
                bt_idx.push_back(make_int4(p0 + a, p0 + b, kd == 1 ? p0 + c : p0 + b, kd));
                bt_par.push_back(make_double2(btk0->as<double>()[t], btx0->as<double>()[t]));
            }
        hr.bt1 = (int)bt_idx.size();
        // bonded partners whose LJ the reference adds in the SR loop and subtracts in
        // polymer_constraints (E:948, E:1132): one entry per subtraction
        for (int64_t t = 0; t < nbt; ++t) {
            const int kd = btk->as<int32_t>()[t];
            const int a = p0 + bta->as<int32_t>()[t];
            const int b = p0 + (kd == 1 ? btc->as<int32_t>()[t] : btb->as<int32_t>()[t]);
            for (int side = 0; side < 2; ++side) {
                const int self = side ? b : a, other = side ? a : b;
                if ((int)excl_of[self].size() >= tis::kExcl)
                    return bail(fail(TIS_ERR_ARG, "replica %d: particle %d has more than %d bonded partners", base + r, self - p0, tis::kExcl));
                excl_of[self].push_back(other);
            }
        }

        // stacks
        const tis::Array *s3E = need(s, "st3_E", base + r, TIS_F64), *s2E = need(s, "st2_E", base + r, TIS_F64);
        if (!s3E || !s2E) return bail(TIS_ERR_ARG);
        const int64_t n3 = s3E->count(), n2 = s2E->count();
        const tis::Array *s3i = need(s, "st3_idx", base + r, TIS_I32, 6 * n3), *s3n = need(s, "st3_native", base + r, TIS_F64, 6 * n3);
        const tis::Array *s2i = need(s, "st2_idx", base + r, TIS_I32, 7 * n2), *s2r = need(s, "st2_r0", base + r, TIS_F64, n2);
        if (!s3i || !s3n || !s2i || !s2r) return bail(TIS_ERR_ARG);
        std::vector<int> off3(2 * n3, -1);
        if (const tis::Array *o = s->get("st3_off")) {
            if (o->dtype != TIS_I32 || o->count() != 2 * n3) return bail(fail(TIS_ERR_ARG, "replica %d: bad st3_off", base + r));
            for (int64_t t = 0; t < 2 * n3; ++t) off3[t] = o->as<int32_t>()[t];
        } else {  // E:1960-1981: a site with ST_EXCESS == 1 switches off stack s3_N + ceil(site/2) - 1
            const tis::Array *site = need(s, "st3_site", base + r, TIS_I32, 2 * n3);
            const tis::Array *exc = need(s, "st_excess", base + r, TIS_I32);
            if (!site || !exc) return bail(TIS_ERR_ARG);
            for (int64_t t = 0; t < 2 * n3; ++t) {
                const int e = site->as<int32_t>()[t];
                if (e >= 1 && e <= exc->count() && exc->as<int32_t>()[e - 1] == 1) {
                    const int idx = (int)ceil(0.5 * e) - 2;
                    if (idx >= 0 && idx < n2) off3[t] = idx;
                }
            }
        }
        hr.s30 = (int)st3_E.size();
        for (int64_t k = 0; k < n3; ++k) {
            for (int c = 0; c < 6; ++c) {
                const int v = s3i->as<int32_t>()[6 * k + c];
                if (v < 0 || v >= nrna) return bail(fail(TIS_ERR_ARG, "replica %d: tertiary stack %lld bad index", base + r, (long long)k));
                st3_idx.push_back(p0 + v);
                st3_nat.push_back(s3n->as<double>()[6 * k + c]);
            }
            st3_E.push_back(s3E->as<double>()[k]);
            st3_off.push_back(off3[2 * k]);
            st3_off.push_back(off3[2 * k + 1]);
        }
        hr.s31 = (int)st3_E.size();
        hr.s20 = (int)st2_E.size();
        const tis::Array *s2d = s->get("st2_dss"), *s2c = s->get("st2_cls");
        const bool have_dss = s2d && s2d->dtype == TIS_F64 && s2d->count() == n2 && s2c && s2c->dtype == TIS_I32 &&
                              s2c->count() == n2;
        for (int64_t k = 0; k < n2; ++k) {
            st2_dss.push_back(have_dss ? s2d->as<double>()[k] : 0.0);
            st2_cls.push_back(have_dss ? s2c->as<int32_t>()[k] : -1);
            for (int c = 0; c < 7; ++c) {
                const int v = s2i->as<int32_t>()[7 * k + c];
                if (v < 0 || v >= nrna) return bail(fail(TIS_ERR_ARG, "replica %d: secondary stack %lld bad index", base + r, (long long)k));
                st2_idx.push_back(p0 + v);
            }
            st2_r0.push_back(s2r->as<double>()[k]);
            st2_E.push_back(s2E->as<double>()[k]);
        }
        hr.s21 = (int)st2_E.size();

        // hydrogen bonds
        const tis::Array *hE = need(s, "hb_E", base + r, TIS_F64);
        const tis::Array *hv = need(s, "hba_valence", base + r, TIS_I32);
        if (!hE || !hv) return bail(TIS_ERR_ARG);
        const int64_t nh = hE->count(), na = hv->count();
        const tis::Array *hi = need(s, "hb_idx", base + r, TIS_I32, 6 * nh), *hn = need(s, "hb_native", base + r, TIS_F64, 6 * nh);
        const tis::Array *hd = need(s, "hb_dode", base + r, TIS_I32, nh), *hao = need(s, "hb_atom_off", base + r, TIS_I32, nh + 1);
        const tis::Array *hco = need(s, "hba_cand_off", base + r, TIS_I32, na + 1);
        if (!hi || !hn || !hd || !hao || !hco) return bail(TIS_ERR_ARG);
        const tis::Array *hai = need(s, "hb_atom_idx", base + r, TIS_I32, hao->as<int32_t>()[nh]);
        const tis::Array *hci = need(s, "hba_cand_idx", base + r, TIS_I32, hco->as<int32_t>()[na]);
        if (!hai || !hci) return bail(TIS_ERR_ARG);
        hr.hb0 = (int)hb_E.size();
        hr.hba0 = (int)hba_val.size();
        const tis::Array *hds = s->get("hb_dhs");
        const bool have_dhs = hds && hds->dtype == TIS_F64 && hds->count() == nh;
        const double hs_D = scalar_f64(s, "hs_D", 0.0);
        for (int64_t k = 0; k < nh; ++k) {
            // hb_E = -0.73753 hs_D per bond of the candidate (E:3881, E:3963)
            hb_dhs.push_back(have_dhs ? hds->as<double>()[k] : hs_D != 0.0 ? hE->as<double>()[k] / hs_D : 0.0);
            for (int c = 0; c < 6; ++c) {
                const int v = hi->as<int32_t>()[6 * k + c];
                if (v < 0 || v >= nrna) return bail(fail(TIS_ERR_ARG, "replica %d: H-bond candidate %lld bad index", base + r, (long long)k));
                hb_idx.push_back(p0 + v);
                hb_nat.push_back(hn->as<double>()[6 * k + c]);
            }
            hb_E.push_back(hE->as<double>()[k]);
            hb_dode.push_back(hd->as<int32_t>()[k]);
            for (int u = hao->as<int32_t>()[k]; u < hao->as<int32_t>()[k + 1]; ++u) {
                const int a = hai->as<int32_t>()[u];
                if (a < 0 || a >= na) return bail(fail(TIS_ERR_ARG, "replica %d: H-bond atom index out of range", base + r));
                hb_aidx.push_back(hr.hba0 + a);
            }
            hb_aoff.push_back((int)hb_aidx.size());
        }
        hr.hb1 = (int)hb_E.size();
        int maxk = 1;
        R.ca0 = (int)ca_list.size();
        for (int64_t a = 0; a < na; ++a) {
            const int v = hv->as<int32_t>()[a];
            hba_val.push_back(v);
            const int cnt = hco->as<int32_t>()[a + 1] - hco->as<int32_t>()[a];
            hba_n.push_back(cnt);
            maxk = std::max(maxk, cnt);
            for (int u = hco->as<int32_t>()[a]; u < hco->as<int32_t>()[a + 1]; ++u) {
                const int k = hci->as<int32_t>()[u];
                if (k < 0 || k >= nh) return bail(fail(TIS_ERR_ARG, "replica %d: H-bond candidate index out of range", base + r));
                hba_cidx.push_back(hr.hb0 + k);
            }
            hba_coff.push_back((int)hba_cidx.size());
            if (cnt > v) ca_list.push_back(hr.hba0 + (int)a);  // only these can exceed their valence
        }
        R.ca1 = (int)ca_list.size();
        hr.hba1 = (int)hba_val.size();
        R.bt0 = hr.bt0; R.bt1 = hr.bt1; R.s30 = hr.s30; R.s31 = hr.s31; R.s20 = hr.s20; R.s21 = hr.s21;
        R.hb0 = hr.hb0; R.hb1 = hr.hb1; R.hba0 = hr.hba0; R.hba1 = hr.hba1;
        R.kscr0 = kscr;
        R.pk0 = h->npk;
        h->npk += n;
        R.maxk = maxk;
        kscr += maxk;
        h->rep.push_back(hr);
        p0 += hr.npad;
        c0 += hr.nc;
    }
    h->P = p0;
    h->C = c0;
    h->nblk = p0 / tis::kBlock;

    // neighbour capacities: ten times the homogeneous expectation, at least 128 / 96
    const double pi = 3.14159265358979323846;
    double rmax_lr = 0;
    for (auto &R : rp) rmax_lr = std::max(rmax_lr, sqrt(R.r2lr));
    const double rsr = prm.sr + prm.skin;
    int cap_sr = prm.cap_sr > 0 ? round_up(prm.cap_sr, 4) : std::max(128, round_up((int)(10 * max_rho * 4.0 / 3.0 * pi * rsr * rsr * rsr), 32));
    int cap_lr = prm.cap_lr > 0 ? round_up(prm.cap_lr, 4)
                                : std::max(96, round_up((int)(10 * max_rho_ch * 4.0 / 3.0 * pi * rmax_lr * rmax_lr * rmax_lr), 32));

    tis::Dev &d = h->dev;
    d.R = h->R;
    d.P = h->P;
    d.nblk = h->nblk;
    d.C = h->C;
    d.fp64 = prm.precision == TIS_PREC_FP64;
    d.full_lists = prm.full_lists ? 1 : 0;
    d.lanes_sr = prm.lanes_sr;
    d.lanes_lr = prm.lanes_lr;
    d.noise = prm.noise;
    d.cap_sr = cap_sr;
    d.cap_lr = cap_lr;
    {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, prm.device);
        d.search_warps = std::max(4, sms * 4);  // one block of 4 warps per SM: rebuilds are rare
        d.sm_count = std::max(1, sms);
        int nc_max = 1;
        for (auto &Q : rp) nc_max = std::max(nc_max, Q.nc);
        d.nc_max = nc_max;
        d.cell_smem = 8 * nc_max <= 160 * 1024 ? 8 * nc_max : 0;  // count/first slot and fill counter per cell
    }
    auto &O = h->owned;
    int rc = TIS_OK;
    std::vector<int4> q(h->P);
    for (int i = 0; i < h->P; ++i) q[i] = make_int4(0, 0, 0, code[i]);
    std::vector<tis::RepState> rs(h->R);
    memset(rs.data(), 0, sizeof(tis::RepState) * h->R);
    for (auto &s : rs) s.lr_now = 1;
    tis::RepParams *d_rp = nullptr;
    tis::RepState *d_rs = nullptr;
    int *d_blk = nullptr, *d_rep = nullptr, *d_cellrep = nullptr;
    int4 *d_q = nullptr;
    if ((rc = dupload(O, &d_rp, rp)) || (rc = dupload(O, &d_rs, rs)) || (rc = dupload(O, &d_blk, blk_rep)) ||
        (rc = dupload(O, &d_rep, rep_of)) || (rc = dupload(O, &d_cellrep, cell_rep)) || (rc = dupload(O, &d_q, q)))
        return bail(rc);
    d.rp = d_rp; d.rs = d_rs; d.blk_rep = d_blk; d.rep_of = d_rep; d.cell_rep = d_cellrep; d.q = d_q;
    {
        excl_of.resize(h->P);
        std::vector<int> ex((size_t)tis::kExcl * h->P, -1), nex(h->P, 0);
        for (int p = 0; p < h->P; ++p) {
            nex[p] = (int)excl_of[p].size();
            for (int k = 0; k < nex[p]; ++k) ex[(size_t)k * h->P + p] = excl_of[p][k];
        }
        int *d_ex = nullptr, *d_nex = nullptr;
        if ((rc = dupload(O, &d_ex, ex)) || (rc = dupload(O, &d_nex, nex))) return bail(rc);
        d.excl = d_ex;
        d.n_excl = d_nex;
    }
    double **sd[9] = {&d.x, &d.y, &d.z, &d.xo, &d.yo, &d.zo, &d.vx, &d.vy, &d.vz};
    for (int c = 0; c < 9; ++c)
        if ((rc = dupload(O, sd[c], st[c]))) return bail(rc);
    if ((rc = dalloc(O, &d.f, 3 * (size_t)h->P)) || (rc = dalloc(O, &d.flr, 3 * (size_t)h->P)) ||
        (rc = dalloc(O, &d.gnoise, (size_t)h->R * tis::kNoise)) || (rc = dalloc(O, &d.cell_of, h->P)) ||
        (rc = dalloc(O, &d.cell_count, h->C)) || (rc = dalloc(O, &d.cell_start, h->C)) ||
        (rc = dalloc(O, &d.cell_fill, h->C)) || (rc = dalloc(O, &d.cell_list, h->P)) || (rc = dalloc(O, &d.qs, h->P)) ||
        (rc = dalloc(O, &d.n_sr, h->P)) || (rc = dalloc(O, &d.n_lr, h->P)) ||
        (rc = dalloc(O, &d.nbr_sr, (size_t)cap_sr * h->P)) || (rc = dalloc(O, &d.nbr_lr, (size_t)cap_lr * h->P)) ||
        (rc = dalloc(O, &d.eterm, (size_t)h->R * tis::kNE)) || (rc = dalloc(O, &d.shift, (size_t)h->R * 3)) || 
        (rc = dalloc(O, &h->d_scalar, 4)) || (rc = dalloc(O, &h->stage, 9 * (size_t)h->npk)) ||
        (rc = dalloc(O, &h->d_e5, 5 * (size_t)h->R)) || (rc = dalloc(O, &h->d_peaks, 2)))
        return bail(rc);
    int4 *d_bti = nullptr;
    double2 *d_btp = nullptr;
    int *i3 = nullptr, *o3 = nullptr, *i2 = nullptr, *ih = nullptr, *dh = nullptr, *ao = nullptr, *ai = nullptr;
    int *hv = nullptr, *co = nullptr, *ci = nullptr, *hn = nullptr, *ca = nullptr;
    double *n3 = nullptr, *e3 = nullptr, *r2 = nullptr, *e2 = nullptr, *nh = nullptr, *eh = nullptr;
    if ((rc = dupload(O, &d_bti, bt_idx)) || (rc = dupload(O, &d_btp, bt_par)) || (rc = dupload(O, &i3, st3_idx)) ||
        (rc = dupload(O, &n3, st3_nat)) || (rc = dupload(O, &e3, st3_E)) || (rc = dupload(O, &o3, st3_off)) ||
        (rc = dupload(O, &i2, st2_idx)) || (rc = dupload(O, &r2, st2_r0)) || (rc = dupload(O, &e2, st2_E)) ||
        (rc = dupload(O, &ih, hb_idx)) || (rc = dupload(O, &nh, hb_nat)) || (rc = dupload(O, &eh, hb_E)) ||
        (rc = dupload(O, &dh, hb_dode)) || (rc = dupload(O, &ao, hb_aoff)) || (rc = dupload(O, &ai, hb_aidx)) ||
        (rc = dupload(O, &hv, hba_val)) || (rc = dupload(O, &co, hba_coff)) || (rc = dupload(O, &ci, hba_cidx)) ||
        (rc = dupload(O, &hn, hba_n)) || (rc = dupload(O, &ca, ca_list)) ||
        (rc = dupload(O, &h->a_st2_dss, st2_dss)) || (rc = dupload(O, &h->a_st2_cls, st2_cls)) ||
        (rc = dupload(O, &h->a_hb_dhs, hb_dhs)))
        return bail(rc);
    d.bt_idx = d_bti; d.bt_par = d_btp;
    d.st3_idx = i3; d.st3_nat = n3; d.st3_E = e3; d.st3_off = o3;
    d.st2_idx = i2; d.st2_r0 = r2; d.st2_E = e2;
    d.hb_idx = ih; d.hb_nat = nh; d.hb_E = eh; d.hb_dode = dh; d.hb_aoff = ao; d.hb_aidx = ai;
    d.hba_val = hv; d.hba_coff = co; d.hba_cidx = ci; d.hba_n = hn; d.ca_list = ca;
    const size_t nst2 = st2_E.size(), nst3 = st3_E.size(), nhb = hb_E.size(), nhba = hba_val.size();
    h->nhb_all = (int)nhb;
    h->nhba_all = (int)nhba;
    d.nbt = (int)bt_idx.size();
    d.nst3 = (int)nst3;
    d.nst2 = (int)nst2;
    {  // secondary stack -> the tertiary stacks whose site can switch it off (E:1960-1981)
        std::vector<std::vector<int>> offby(nst2);
        for (int r = 0; r < h->R; ++r)
            for (int k = h->rep[r].s30; k < h->rep[r].s31; ++k)
                for (int sd = 0; sd < 2; ++sd) {
                    const int t = st3_off[2 * k + sd];
                    if (t >= 0) offby[h->rep[r].s20 + t].push_back(k);
                }
        std::vector<int> off{0}, idx;
        for (auto &v : offby) {
            for (int k : v) idx.push_back(k);
            off.push_back((int)idx.size());
        }
        int *d_off = nullptr, *d_idx = nullptr;
        if ((rc = dupload(O, &d_off, off)) || (rc = dupload(O, &d_idx, idx))) return bail(rc);
        d.st2_offby_off = d_off;
        d.st2_offby_idx = d_idx;
    }
    if ((rc = dalloc(O, &d.st_energy, nst3)) ||
        (rc = dalloc(O, &d.hb_status, nhb)) || (rc = dalloc(O, &d.hb_excess, nhba)) ||
        (rc = dalloc(O, &d.hb_active, nhb)) || (rc = dalloc(O, &d.ca_exc, ca_list.size())) ||
        (rc = dalloc(O, &d.hb_K, (size_t)kscr)) || (rc = dalloc(O, &d.hb_A, ca_list.size())) ||
        (rc = dalloc(O, &d.hb_energy, nhb)) || (rc = dalloc(O, &d.hb_code, nhb)) ||
        (rc = dalloc(O, &d.hb_term, 6 * nhb)) || (rc = dalloc(O, &d.hb_br, 3 * nhb)))
        return bail(rc);
    {  // the Monte Carlo's views of the candidates: per over-valence atom its candidates, per candidate its such atoms
        std::vector<int> ca_pos(nhba, -1), ca_coff{0}, ca_cidx, hb_coff{0}, hb_cpos;
        int hb_nmax = 0, ca_nmax = 0, k_nmax = 0, cidx_max = 0, cpos_max = 0;
        for (int r = 0; r < h->R; ++r) {
            const tis::RepParams &Q = rp[r];
            const size_t c_first = ca_cidx.size();
            for (int i = Q.ca0; i < Q.ca1; ++i) {
                const int a = ca_list[i];
                ca_pos[a] = i - Q.ca0;
                for (int t = hba_coff[a]; t < hba_coff[a + 1]; ++t) ca_cidx.push_back(hba_cidx[t] - Q.hb0);
                ca_coff.push_back((int)ca_cidx.size());
            }
            cidx_max = std::max(cidx_max, (int)(ca_cidx.size() - c_first));
            hb_nmax = std::max(hb_nmax, Q.hb1 - Q.hb0);
            ca_nmax = std::max(ca_nmax, Q.ca1 - Q.ca0);
            k_nmax = std::max(k_nmax, Q.maxk);
        }
        for (int r = 0; r < h->R; ++r) {
            const size_t p_first = hb_cpos.size();
            for (int k = rp[r].hb0; k < rp[r].hb1; ++k) {
                for (int u = hb_aoff[k]; u < hb_aoff[k + 1]; ++u)
                    if (ca_pos[hb_aidx[u]] >= 0) hb_cpos.push_back(ca_pos[hb_aidx[u]]);
                hb_coff.push_back((int)hb_cpos.size());
            }
            cpos_max = std::max(cpos_max, (int)(hb_cpos.size() - p_first));
        }
        int *d1 = nullptr, *d2 = nullptr, *d3 = nullptr, *d4 = nullptr;
        if ((rc = dupload(O, &d1, ca_coff)) || (rc = dupload(O, &d2, ca_cidx)) || (rc = dupload(O, &d3, hb_coff)) ||
            (rc = dupload(O, &d4, hb_cpos)))
            return bail(rc);
        d.ca_coff = d1; d.ca_cidx = d2; d.hb_coff = d3; d.hb_cpos = d4;
        d.hb_nmax = hb_nmax;
        d.ca_nmax = ca_nmax;
        d.k_nmax = k_nmax;
        d.cidx_max = cidx_max;
        d.cpos_max = cpos_max;
        const size_t smem = tis::hb_layout(hb_nmax, ca_nmax, k_nmax, cidx_max, cpos_max).total;
        d.hb_smem = smem <= 160 * 1024 ? (int)smem : 0;
    }
    if (tis::configure_kernels(d) != 0) return bail(fail(TIS_ERR_CUDA, "cudaFuncSetAttribute failed"));
    if (cudaMallocHost((void **)&h->h_rs, sizeof(tis::RepState) * h->R) != cudaSuccess ||
        cudaMallocHost((void **)&h->h_peaks, 2 * sizeof(int)) != cudaSuccess)
        return bail(fail(TIS_ERR_NOMEM, "cudaMallocHost failed"));
    // the allocations' memsets and the pageable uploads above run on the legacy
    // default stream, which the group's non-blocking streams do not wait for
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(fail(TIS_ERR_CUDA, "device synchronisation failed"));
    tis::launch_quantize(h->dev, h->stream);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(h->stream) != cudaSuccess)
        return bail(fail(TIS_ERR_CUDA, "quantisation kernel failed"));
    *out = h;
    return TIS_OK;
}

static int grp_destroy(Group *h)
{
    if (h) {
        cudaSetDevice(h->prm.device);
        cudaStreamSynchronize(h->stream);
        delete h;
    }
    return TIS_OK;
}

static int grp_set_state(Group *h, int r, const double *x, const double *y, const double *z, const double *xo,
                  const double *yo, const double *zo, const double *vx, const double *vy, const double *vz)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    const double *src[9] = {x, y, z, xo, yo, zo, vx, vy, vz};
    double *dst[9] = {h->dev.x, h->dev.y, h->dev.z, h->dev.xo, h->dev.yo, h->dev.zo, h->dev.vx, h->dev.vy, h->dev.vz};
    const RepHost &hr = h->rep[r];
    for (int c = 0; c < 9; ++c) {
        if (!src[c]) return fail(TIS_ERR_ARG, "tis_set_state: null array %d", c);
        TIS_CUDA(cudaMemcpyAsync(dst[c] + hr.p0, src[c], sizeof(double) * hr.n, cudaMemcpyHostToDevice, h->stream));
    }
    tis::launch_quantize(h->dev, h->stream);
    TIS_CUDA(cudaGetLastError());
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    h->lists_built = false;
    return TIS_OK;
}

static int grp_get_state(Group *h, int r, double *x, double *y, double *z, double *xo, double *yo, double *zo,
                  double *vx, double *vy, double *vz)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    double *dst[9] = {x, y, z, xo, yo, zo, vx, vy, vz};
    double *src[9] = {h->dev.x, h->dev.y, h->dev.z, h->dev.xo, h->dev.yo, h->dev.zo, h->dev.vx, h->dev.vy, h->dev.vz};
    const RepHost &hr = h->rep[r];
    for (int c = 0; c < 9; ++c)
        if (dst[c]) TIS_CUDA(cudaMemcpyAsync(dst[c], src[c] + hr.p0, sizeof(double) * hr.n, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return TIS_OK;
}

static int grp_get_all_energies(Group *h, double *out)
{
    tis::launch_energies(h->dev, h->stream, h->d_e5);
    TIS_CUDA(cudaGetLastError());
    TIS_CUDA(cudaMemcpyAsync(out, h->d_e5, sizeof(double) * 5 * h->R, cudaMemcpyDeviceToHost, h->stream));
    return TIS_OK;
}


static int grp_get_cells(Group *h, int r, int32_t *cell, int32_t *dims)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    const RepHost &hr = h->rep[r];
    if (cell) TIS_CUDA(cudaMemcpyAsync(cell, h->dev.cell_of + hr.p0, sizeof(int) * hr.n, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    if (dims) for (int k = 0; k < 3; ++k) dims[k] = hr.mc[k];
    return TIS_OK;
}

static int grp_get_pairs(Group *h, int r, int which, int32_t *pairs, int64_t cap, int64_t *n)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    const RepHost &hr = h->rep[r];
    const int capl = which ? h->dev.cap_lr : h->dev.cap_sr;
    const int *nbr = which ? h->dev.nbr_lr : h->dev.nbr_sr;
    const int *cnt = which ? h->dev.n_lr : h->dev.n_sr;
    std::vector<int> c(hr.npad), lst((size_t)capl * hr.npad);
    TIS_CUDA(cudaMemcpyAsync(c.data(), cnt + hr.p0, sizeof(int) * hr.npad, cudaMemcpyDeviceToHost, h->stream));
    // chunk-major slots: chunk k/4 of the replica's particles is 4*npad contiguous ints
    TIS_CUDA(cudaMemcpy2DAsync(lst.data(), sizeof(int) * 4 * hr.npad, nbr + tis::nb_idx(0, hr.p0, h->P),
                               sizeof(int) * 4 * (size_t)h->P, sizeof(int) * 4 * hr.npad, capl / 4,
                               cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    std::vector<std::pair<int, int>> pr;
    for (int i = 0; i < hr.n; ++i)
        for (int k = 0; k < c[i]; ++k) {
            const int j = (lst[tis::nb_idx(k, i, hr.npad)] & tis::kIdxMask) - hr.p0;
            if (i < j) pr.emplace_back(i, j);
        }
    std::sort(pr.begin(), pr.end());
    if (n) *n = 2 * (int64_t)pr.size();
    if (pairs)
        for (int64_t t = 0; t < (int64_t)pr.size() && 2 * t + 1 < cap; ++t) {
            pairs[2 * t] = pr[t].first;
            pairs[2 * t + 1] = pr[t].second;
        }
    return TIS_OK;
}

static int grp_ion_counts(Group *h, int r, int kind, double radius, int32_t *counts, int64_t cap, int64_t *n_p,
                          int32_t *total)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    if (kind != 0 && (kind < 3 || kind > 5))
        return fail(TIS_ERR_ARG, "tis_ion_counts: kind %d is not 0 (P), 3 (Mg), 4 (Cl) or 5 (K)", kind);
    if (!(radius > 0) || radius > h->prm.sr)
        return fail(TIS_ERR_ARG, "tis_ion_counts: radius %g outside (0, %g] (the SR radius)", radius, h->prm.sr);
    if (!h->lists_built && (rc = populate(h))) return rc;
    const RepHost &hr = h->rep[r];
    int *d_cnt = nullptr, *d_hit = nullptr;
    TIS_CUDA(cudaMallocAsync((void **)&d_cnt, sizeof(int) * (hr.nrna + hr.n), h->stream));
    d_hit = d_cnt + hr.nrna;
    TIS_CUDA(cudaMemsetAsync(d_hit, 0, sizeof(int) * hr.n, h->stream));
    tis::launch_ion_counts(h->dev, h->stream, r, hr.nrna, kind, radius * radius, d_cnt, d_hit);
    std::vector<int> c(hr.nrna + hr.n);
    TIS_CUDA(cudaMemcpyAsync(c.data(), d_cnt, sizeof(int) * c.size(), cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaFreeAsync(d_cnt, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    int64_t np = 0;
    for (int i = 0; i < hr.nrna; ++i)
        if (c[i] >= 0) {
            if (counts && np < cap) counts[np] = c[i];
            ++np;
        }
    if (n_p) *n_p = np;
    if (total) {
        int t = 0;
        for (int j = 0; j < hr.n; ++j) t += c[hr.nrna + j];
        *total = t;
    }
    return check_flags(h);
}

static int grp_get_hb_status(Group *h, int r, int32_t *status, int32_t *excess)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    const RepHost &hr = h->rep[r];
    if (status && hr.hb1 > hr.hb0)
        TIS_CUDA(cudaMemcpyAsync(status, h->dev.hb_status + hr.hb0, sizeof(int) * (hr.hb1 - hr.hb0), cudaMemcpyDeviceToHost, h->stream));
    if (excess && hr.hba1 > hr.hba0)
        TIS_CUDA(cudaMemcpyAsync(excess, h->dev.hb_excess + hr.hba0, sizeof(int) * (hr.hba1 - hr.hba0), cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return TIS_OK;
}

static int grp_compute_forces(Group *h, int r, int mask, double *forces, double *energies)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    if (!h->lists_built && (rc = populate(h))) return rc;
    if ((rc = clear_flags(h))) return rc;
    const tis::Dev &d = h->dev;
    TIS_CUDA(cudaMemsetAsync(d.eterm, 0, sizeof(double) * h->R * tis::kNE, h->stream));
    TIS_CUDA(cudaMemsetAsync(d.f, 0, sizeof(unsigned long long) * 3 * h->P, h->stream));
    if (mask & TIS_TERM_SR) tis::launch_pair_sr(d, h->stream, true, false);
    if (mask & TIS_TERM_LR) tis::launch_pair_lr(d, h->stream, true, true);
    else TIS_CUDA(cudaMemsetAsync(d.flr, 0, sizeof(unsigned long long) * 3 * h->P, h->stream));
    const int tmask = (mask & TIS_TERM_BONDED ? 4 : 0) | (mask & TIS_TERM_STACK ? 8 : 0) | (mask & TIS_TERM_HB ? 16 : 0);
    if (tmask) tis::launch_topology(d, h->stream, tmask, true, false, false);
    tis::launch_rg(d, h->stream, r, h->d_scalar);
    TIS_CUDA(cudaGetLastError());
    const RepHost &hr = h->rep[r];
    std::vector<unsigned long long> f(3 * (size_t)hr.n), fl(3 * (size_t)hr.n);
    for (int c = 0; c < 3; ++c) {
        TIS_CUDA(cudaMemcpyAsync(f.data() + c * hr.n, d.f + (size_t)c * h->P + hr.p0, 8 * hr.n, cudaMemcpyDeviceToHost, h->stream));
        TIS_CUDA(cudaMemcpyAsync(fl.data() + c * hr.n, d.flr + (size_t)c * h->P + hr.p0, 8 * hr.n, cudaMemcpyDeviceToHost, h->stream));
    }
    double et[tis::kNE], rg = 0;
    tis::RepState st;
    TIS_CUDA(cudaMemcpyAsync(et, d.eterm + r * tis::kNE, sizeof et, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaMemcpyAsync(&rg, h->d_scalar, sizeof rg, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaMemcpyAsync(&st, d.rs + r, sizeof st, cudaMemcpyDeviceToHost, h->stream));
    // the step's force kernels accumulate into a zero sum: leave it so
    TIS_CUDA(cudaMemsetAsync(d.f, 0, sizeof(unsigned long long) * 3 * h->P, h->stream));
    TIS_CUDA(cudaMemsetAsync(d.flr, 0, sizeof(unsigned long long) * 3 * h->P, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    if (forces)
        for (int i = 0; i < hr.n; ++i)
            for (int c = 0; c < 3; ++c) {
                const size_t k = (size_t)c * hr.n + i;
                double v;
                if (d.fp64) {
                    double a, b;
                    memcpy(&a, &f[k], 8);
                    memcpy(&b, &fl[k], 8);
                    v = a + b;
                } else {
                    v = (double)(long long)(f[k] + fl[k]) / tis::kFixScale;
                }
                forces[3 * i + c] = v;
            }
    if (energies) {
        for (int k = 0; k < tis::kNE; ++k) energies[k] = et[k];
        energies[TIS_E_RG] = rg;
    }
    return check_flags(h);
}

// ---------------------------------------------------------------------------
// parameter derivatives and the reverse pass through steps (no counterpart in
// the reference)
// ---------------------------------------------------------------------------
// device memory of one adjoint call, zeroed on the group's stream, freed with it
struct AdjMem {
    std::vector<void *> owned;
    ~AdjMem()
    {
        for (void *p : owned) cudaFree(p);
    }
    template <class T>
    int alloc(Group *h, T **p, size_t count)
    {
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
        if (e != cudaSuccess)
            return fail(TIS_ERR_NOMEM, "cudaMalloc(%zu bytes) for the adjoint: %s", count * sizeof(T), cudaGetErrorString(e));
        owned.push_back((void *)*p);
        e = cudaMemsetAsync(*p, 0, count * sizeof(T), h->stream);
        if (e != cudaSuccess) return fail(TIS_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
        return TIS_OK;
    }
};

static_assert(tis::kNParams == TIS_N_PARAMS, "parameter count");

tis::AdjDev adj_base(const Group *h)
{
    tis::AdjDev a{};
    a.st2_dss = h->a_st2_dss;
    a.st2_cls = h->a_st2_cls;
    a.hb_dhs = h->a_hb_dhs;
    a.nhb = h->nhb_all;
    return a;
}

static int grp_param_grad(Group *h, double *out)
{
    int rc;
    if (!h->lists_built && (rc = populate(h))) return rc;
    if ((rc = clear_flags(h))) return rc;
    AdjMem M;
    tis::AdjDev a = adj_base(h);
    if ((rc = M.alloc(h, &a.dth, (size_t)h->R * tis::kNParams)) || (rc = M.alloc(h, &a.rhb, (size_t)h->nhb_all)))
        return rc;
    const size_t fbytes = sizeof(unsigned long long) * 3 * h->P;
    // the valence-limited Monte Carlo of this state (as a force evaluation runs it),
    // recording the bonds it leaves formed; its forces are dropped
    tis::Dev dr = h->dev;
    dr.hb_rec = a.rhb;
    TIS_CUDA(cudaMemsetAsync(h->dev.f, 0, fbytes, h->stream));
    tis::launch_topology(dr, h->stream, 16, false, false, true);
    TIS_CUDA(cudaMemsetAsync(h->dev.f, 0, fbytes, h->stream));
    a.px = h->dev.x;
    a.py = h->dev.y;
    a.pz = h->dev.z;
    tis::launch_adj_pair(h->dev, a, h->stream, false, nullptr, 0);
    tis::launch_adj_pair(h->dev, a, h->stream, true, nullptr, 0);
    tis::launch_adj_topo(h->dev, a, h->stream, nullptr, 0);
    TIS_CUDA(cudaGetLastError());
    TIS_CUDA(cudaMemcpyAsync(out, a.dth, sizeof(double) * h->R * tis::kNParams, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return check_flags(h);
}

// the device arrays a step reads and leaves for the next one (the rest is rebuilt
// or scratch): a checkpoint holds copies of these
std::vector<std::pair<void *, size_t>> step_state(const Group *h)
{
    const tis::Dev &d = h->dev;
    const size_t P = h->P;
    std::vector<std::pair<void *, size_t>> v;
    for (double *p : {d.x, d.y, d.z, d.xo, d.yo, d.zo, d.vx, d.vy, d.vz}) v.emplace_back(p, 8 * P);
    v.emplace_back(d.q, sizeof(int4) * P);
    v.emplace_back(d.flr, 24 * P);
    v.emplace_back(d.rs, sizeof(tis::RepState) * h->R);
    v.emplace_back(d.n_sr, 4 * P);
    v.emplace_back(d.n_lr, 4 * P);
    v.emplace_back(d.nbr_sr, 4 * (size_t)d.cap_sr * P);
    v.emplace_back(d.nbr_lr, 4 * (size_t)d.cap_lr * P);
    v.emplace_back(d.hb_status, 4 * (size_t)h->nhb_all);
    v.emplace_back(d.hb_excess, 4 * (size_t)h->nhba_all);
    v.emplace_back(d.hb_active, 4 * (size_t)h->nhb_all);
    return v;
}

inline size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// seed: the group's part of nine packed arrays from offset `off` (NULL entries zero);
// dtheta: R x kNParams of the group; dstate0: packed like seed (NULL entries skipped)
static int grp_traj_grad(Group *h, int64_t steps, int K, const double *const *seed, int64_t off, double *dtheta,
                         double *const *dstate0)
{
    int rc;
    if ((rc = clear_flags(h))) return rc;
    if ((rc = populate(h))) return rc;  // the run starts with populate_lists (E:6237): lists and LR force fresh
    const tis::Dev &d = h->dev;
    const size_t P = h->P, R = h->R;
    const auto st = step_state(h);
    size_t sbytes = 0;
    for (const auto &e : st) sbytes += align256(e.second);
    const int64_t nseg = (steps + K - 1) / K;
    AdjMem M;
    char *arena = nullptr;
    tis::AdjDev a = adj_base(h);
    double *rx, *rf, *rg;
    int *rhb, *rlr, *rnsr, *rnlr, *rbsr, *rblr;
    const size_t Kz = (size_t)K, nhb = (size_t)h->nhb_all;
    if ((rc = M.alloc(h, &arena, (size_t)(nseg + 1) * sbytes)) || (rc = M.alloc(h, &a.lam, 9 * P)) ||
        (rc = M.alloc(h, &a.lamf, 3 * P)) || (rc = M.alloc(h, &a.mu, 3 * P)) || (rc = M.alloc(h, &a.jv, 3 * P)) ||
        (rc = M.alloc(h, &a.cen, 3 * R)) || (rc = M.alloc(h, &a.dth, R * tis::kNParams)) ||
        (rc = M.alloc(h, &rx, Kz * 9 * P)) || (rc = M.alloc(h, &rf, Kz * 3 * P)) ||
        (rc = M.alloc(h, &rg, Kz * R * tis::kNoise)) || (rc = M.alloc(h, &rhb, Kz * std::max<size_t>(nhb, 1))) ||
        (rc = M.alloc(h, &rlr, Kz * R)) || (rc = M.alloc(h, &rnsr, Kz * P)) || (rc = M.alloc(h, &rnlr, Kz * P)) ||
        (rc = M.alloc(h, &rbsr, Kz * d.cap_sr * P)) || (rc = M.alloc(h, &rblr, Kz * d.cap_lr * P)))
        return rc;
    auto save = [&](int64_t slot) {
        char *p = arena + slot * sbytes;
        for (const auto &e : st) {
            if (e.second) cudaMemcpyAsync(p, e.first, e.second, cudaMemcpyDeviceToDevice, h->stream);
            p += align256(e.second);
        }
    };
    auto restore = [&](int64_t slot) {
        const char *p = arena + slot * sbytes;
        for (const auto &e : st) {
            if (e.second) cudaMemcpyAsync(e.first, p, e.second, cudaMemcpyDeviceToDevice, h->stream);
            p += align256(e.second);
        }
    };
    // the recorded step j of a segment: its inputs and the lists its forces read
    auto slot = [&](int j, tis::Dev &dj) {
        tis::AdjDev aj = a;
        aj.rx = rx + (size_t)j * 9 * P;
        aj.rf = rf + (size_t)j * 3 * P;
        aj.rg = rg + (size_t)j * R * tis::kNoise;
        aj.rhb = rhb + (size_t)j * std::max<size_t>(nhb, 1);
        aj.rlr = rlr + (size_t)j * R;
        aj.px = aj.rx;
        aj.py = aj.rx + P;
        aj.pz = aj.rx + 2 * P;
        dj = d;
        dj.n_sr = rnsr + (size_t)j * P;
        dj.n_lr = rnlr + (size_t)j * P;
        dj.nbr_sr = rbsr + (size_t)j * d.cap_sr * P;
        dj.nbr_lr = rblr + (size_t)j * d.cap_lr * P;
        return aj;
    };

    // forward, a checkpoint every K steps and one of the final state
    for (int64_t s = 0; s < steps; ++s) {
        if (s % K == 0) save(s / K);
        enqueue_step(h);
    }
    save(nseg);
    TIS_CUDA(cudaGetLastError());
    if ((rc = check_flags(h))) return rc;

    // dL/d(final state)
    unsigned mask = 0;
    for (int c = 0; c < 9; ++c)
        if (seed && seed[c]) {
            mask |= 1u << c;
            TIS_CUDA(cudaMemcpyAsync(h->stage + (size_t)c * h->npk, seed[c] + off, sizeof(double) * h->npk,
                                     cudaMemcpyHostToDevice, h->stream));
        }
    tis::launch_adj_unpack(d, h->stream, a.lam, h->stage, h->npk, mask);

    // backward: each segment recomputed from its checkpoint, then its steps in reverse
    for (int64_t g = nseg - 1; g >= 0; --g) {
        restore(g);
        const int len = (int)std::min<int64_t>(K, steps - g * K);
        for (int j = 0; j < len; ++j) {
            tis::Dev dj;
            const tis::AdjDev aj = slot(j, dj);
            h->dev.hb_rec = aj.rhb;
            enqueue_forces(h, true);
            h->dev.hb_rec = nullptr;
            TIS_CUDA(cudaMemcpyAsync(aj.rg, d.gnoise, sizeof(double) * R * tis::kNoise, cudaMemcpyDeviceToDevice, h->stream));
            TIS_CUDA(cudaMemcpyAsync(dj.n_sr, d.n_sr, 4 * P, cudaMemcpyDeviceToDevice, h->stream));
            TIS_CUDA(cudaMemcpyAsync(dj.n_lr, d.n_lr, 4 * P, cudaMemcpyDeviceToDevice, h->stream));
            TIS_CUDA(cudaMemcpyAsync(dj.nbr_sr, d.nbr_sr, 4 * (size_t)d.cap_sr * P, cudaMemcpyDeviceToDevice, h->stream));
            TIS_CUDA(cudaMemcpyAsync(dj.nbr_lr, d.nbr_lr, 4 * (size_t)d.cap_lr * P, cudaMemcpyDeviceToDevice, h->stream));
            tis::launch_adj_record(d, aj, h->stream);
            tis::launch_integrate(d, h->stream);
            tis::launch_rebuild(d, h->stream);
        }
        for (int j = len - 1; j >= 0; --j) {
            tis::Dev dj;
            const tis::AdjDev aj = slot(j, dj);
            tis::launch_adj_step(dj, aj, h->stream);
        }
        TIS_CUDA(cudaGetLastError());
    }
    if ((rc = check_flags(h))) return rc;
    restore(nseg);
    TIS_CUDA(cudaMemcpyAsync(dtheta, a.dth, sizeof(double) * R * tis::kNParams, cudaMemcpyDeviceToHost, h->stream));
    if (dstate0) {
        tis::launch_adj_pack(d, h->stream, a.lam, h->stage, h->npk);
        for (int c = 0; c < 9; ++c)
            if (dstate0[c])
                TIS_CUDA(cudaMemcpyAsync(dstate0[c] + off, h->stage + (size_t)c * h->npk, sizeof(double) * h->npk,
                                         cudaMemcpyDeviceToHost, h->stream));
    }
    TIS_CUDA(cudaGetLastError());
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return check_flags(h);
}

static int grp_deterministic_forces(Group *h)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    int rc;
    if (!h->lists_built && (rc = populate(h))) return rc;
    // E:2532: the force sum starts from zero (the fused step's integrator leaves it zero)
    TIS_CUDA(cudaMemsetAsync(h->dev.f, 0, sizeof(unsigned long long) * 3 * h->P, h->stream));
    enqueue_forces(h, false);
    TIS_CUDA(cudaGetLastError());
    return TIS_OK;
}

static int grp_get_forces(Group *h, int r, double *forces)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    if (!forces) return fail(TIS_ERR_ARG, "null output");
    const RepHost &hr = h->rep[r];
    const tis::Dev &d = h->dev;
    std::vector<unsigned long long> f(3 * (size_t)hr.n), fl(3 * (size_t)hr.n);
    for (int c = 0; c < 3; ++c) {
        TIS_CUDA(cudaMemcpyAsync(f.data() + c * hr.n, d.f + (size_t)c * h->P + hr.p0, 8 * hr.n, cudaMemcpyDeviceToHost, h->stream));
        TIS_CUDA(cudaMemcpyAsync(fl.data() + c * hr.n, d.flr + (size_t)c * h->P + hr.p0, 8 * hr.n, cudaMemcpyDeviceToHost, h->stream));
    }
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < hr.n; ++i)
        for (int c = 0; c < 3; ++c) {
            const size_t k = (size_t)c * hr.n + i;
            if (d.fp64) {
                double a, b;
                memcpy(&a, &f[k], 8);
                memcpy(&b, &fl[k], 8);
                forces[3 * i + c] = a + b;
            } else {
                forces[3 * i + c] = (double)(long long)(f[k] + fl[k]) / tis::kFixScale;
            }
        }
    return check_flags(h);
}

static int grp_full_forces(Group *h)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    tis::launch_noise(h->dev, h->stream);
    TIS_CUDA(cudaGetLastError());
    return TIS_OK;
}

static int grp_move_rigid_units(Group *h)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    tis::launch_integrate(h->dev, h->stream);
    TIS_CUDA(cudaGetLastError());
    return TIS_OK;
}

static int grp_check_shifts(Group *h)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    // the displacement check itself ran at the end of tis_move_rigid_units
    tis::launch_rebuild(h->dev, h->stream);
    TIS_CUDA(cudaGetLastError());
    return TIS_OK;
}

static int grp_step(Group *h, int64_t n)
{
    if (!h || n < 0) return fail(TIS_ERR_ARG, "tis_step: bad argument");
    int rc;
    if (!h->lists_built && (rc = populate(h))) return rc;
    int64_t left = n;
    if (h->prm.use_graph && n >= h->prm.graph_steps) {
        if (!h->graph) {
            if ((rc = capture_steps(h, h->prm.graph_steps, &h->graph))) return rc;
            h->graph_steps = h->prm.graph_steps;
        }
        while (left >= h->graph_steps) {
            TIS_CUDA(cudaGraphLaunch(h->graph, h->stream));
            left -= h->graph_steps;
        }
    }
    if (h->prm.use_graph && left > 0) {
        // the remainder runs from a graph of its own length, kept for the next call
        // with the same remainder (a caller stepping by a fixed count below the graph
        // length replays it every call)
        if (!h->tail || h->tail_steps != left) {
            TIS_CUDA(cudaStreamSynchronize(h->stream));  // the old remainder graph may still run
            if (h->tail) cudaGraphExecDestroy(h->tail);
            h->tail = nullptr;
            h->tail_steps = 0;
            if ((rc = capture_steps(h, (int)left, &h->tail))) return rc;
            h->tail_steps = (int)left;
        }
        TIS_CUDA(cudaGraphLaunch(h->tail, h->stream));
        left = 0;
    }
    for (int64_t s = 0; s < left; ++s) enqueue_step(h);
    TIS_CUDA(cudaGetLastError());
    h->launches += n * tis::kernel_launches_per_step();
    return TIS_OK;
}

static int grp_profile_stages(Group *h, int64_t n, double *ms)
{
    if (!h || n < 1 || !ms) return fail(TIS_ERR_ARG, "tis_profile_stages: bad argument");
    int rc;
    if (!h->lists_built && (rc = populate(h))) return rc;
    constexpr int kS = TIS_N_STAGES;
    cudaEvent_t ev[kS + 1];
    for (auto &e : ev) TIS_CUDA(cudaEventCreate(&e));
    double acc[kS] = {};
    const tis::Dev &d = h->dev;
    for (int64_t s = 0; s < n; ++s) {
        TIS_CUDA(cudaEventRecord(ev[0], h->stream));
        tis::launch_pair_sr(d, h->stream, false, true);
        TIS_CUDA(cudaEventRecord(ev[1], h->stream));
        tis::launch_pair_lr(d, h->stream, false, false);
        TIS_CUDA(cudaEventRecord(ev[2], h->stream));
        tis::launch_topology(d, h->stream, 4 | 8, false, false, true);
        TIS_CUDA(cudaEventRecord(ev[3], h->stream));
        tis::launch_topology(d, h->stream, 16, false, true, true);
        TIS_CUDA(cudaEventRecord(ev[4], h->stream));
        tis::launch_shift(d, h->stream);
        TIS_CUDA(cudaEventRecord(ev[5], h->stream));
        tis::launch_move(d, h->stream);  // the skin check runs in its last blocks
        TIS_CUDA(cudaEventRecord(ev[6], h->stream));
        tis::launch_cells(d, h->stream);
        TIS_CUDA(cudaEventRecord(ev[7], h->stream));
        tis::launch_search(d, h->stream);
        TIS_CUDA(cudaEventRecord(ev[8], h->stream));
        TIS_CUDA(cudaEventSynchronize(ev[kS]));
        for (int k = 0; k < kS; ++k) {
            float t = 0;
            TIS_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            acc[k] += t;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int k = 0; k < kS; ++k) ms[k] = acc[k] / (double)n;
    h->launches += n * tis::kernel_launches_per_step();
    return check_flags(h);
}

static int grp_sync(Group *h)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    return check_flags(h);
}

static int grp_get_energies(Group *h, int r, double *out5)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    if (!out5) return fail(TIS_ERR_ARG, "null output");
    tis::RepState st;
    double rg = 0;
    tis::launch_rg(h->dev, h->stream, r, h->d_scalar);
    TIS_CUDA(cudaMemcpyAsync(&st, h->dev.rs + r, sizeof st, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaMemcpyAsync(&rg, h->d_scalar, sizeof rg, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    out5[0] = st.e2hb;
    out5[1] = st.e3hb;
    out5[2] = st.e2st;
    out5[3] = st.e3st;
    out5[4] = rg;
    return TIS_OK;
}

static int grp_get_stack_energies(Group *h, int r, double *out, int64_t cap, int64_t *n)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    const RepHost &hr = h->rep[r];
    const int64_t m = hr.s31 - hr.s30;
    if (n) *n = m;
    if (out && m > 0)
        TIS_CUDA(cudaMemcpyAsync(out, h->dev.st_energy + hr.s30, sizeof(double) * std::min(m, cap), cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return TIS_OK;
}

static int grp_get_counters(Group *h, int r, int64_t *klok, int64_t *rebuilds, int64_t *draws)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    tis::RepState st;
    TIS_CUDA(cudaMemcpyAsync(&st, h->dev.rs + r, sizeof st, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    if (klok) *klok = st.klok;
    if (rebuilds) *rebuilds = st.rebuilds;
    if (draws) *draws = (int64_t)st.ctr;
    return TIS_OK;
}

static int grp_replica_size(Group *h, int r, int *n_particles)
{
    int rc = valid_replica(h, r);
    if (rc) return rc;
    if (n_particles) *n_particles = h->rep[r].n;
    return TIS_OK;
}


// The public handle: replicas split into groups of consecutive replicas.  Each
// group's work is forked from and joined back into the handle's stream, so the
// groups' kernels overlap on the GPU while calls stay ordered on one stream.
struct tis_handle {
    int R = 0;
    tis_run_params prm{};
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<Group *> groups;
    std::vector<cudaEvent_t> join;
    std::vector<int> grp_of, loc_of;
    std::vector<tis_density *> densities;  // grids on this handle: released with it
    // step graphs of the whole handle (every group's branch, forked from and joined
    // into the handle's stream): the graph length and the last remainder length
    struct StepGraph {
        int steps = 0;
        cudaGraphExec_t exec = nullptr;
        std::vector<long long> gens;  // the groups' list generations it was captured with
    };
    StepGraph full, tail;
    tis_frame_ring *ring = nullptr;  // frames written from inside the step (tis_frames_start)
    int64_t npk = 0;                 // particles of all replicas (unpadded)
    double *stage = nullptr;         // nine packed state arrays of npk values (tis_set_states / tis_get_states)

    ~tis_handle()
    {
        if (stream) cudaStreamSynchronize(stream);  // graphs launched on it may still use the groups' memory
        if (stage) cudaFree(stage);
        for (StepGraph *sg : {&full, &tail})
            if (sg->exec) cudaGraphExecDestroy(sg->exec);
        for (Group *g : groups) delete g;
        for (cudaEvent_t e : join) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// the groups' streams wait for the work queued so far on the handle's stream
int fork_groups(tis_handle *h)
{
    TIS_CUDA(cudaEventRecord(h->fork, h->stream));
    for (Group *g : h->groups) TIS_CUDA(cudaStreamWaitEvent(g->stream, h->fork, 0));
    return TIS_OK;
}

// the handle's stream waits for everything queued on the groups' streams
int join_groups(tis_handle *h)
{
    for (size_t k = 0; k < h->groups.size(); ++k) {
        TIS_CUDA(cudaEventRecord(h->join[k], h->groups[k]->stream));
        TIS_CUDA(cudaStreamWaitEvent(h->stream, h->join[k], 0));
    }
    return TIS_OK;
}

// runs fn on every group between a fork and a join; stops at the first error
template <class F>
int each_group(tis_handle *h, F fn)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    int rc = fork_groups(h);
    for (size_t k = 0; k < h->groups.size() && rc == TIS_OK; ++k) rc = fn(h->groups[k]);
    const int rj = join_groups(h);
    return rc ? rc : rj;
}

// populate_lists for the given groups, ordered after the work queued on the
// handle's stream: every group's build is launched before any is checked, so the
// builds overlap; groups whose lists had to grow build again
int populate_groups(tis_handle *h, std::vector<Group *> pending)
{
    int rc = fork_groups(h);
    if (rc) return rc;
    for (int attempt = 0; !pending.empty(); ++attempt) {
        for (Group *g : pending)
            if ((rc = populate_launch(g))) return rc;
        std::vector<Group *> again_list;
        for (Group *g : pending) {
            TIS_CUDA(cudaStreamSynchronize(g->stream));
            bool again = false;
            if ((rc = populate_check(g, attempt, &again))) return rc;
            if (again) again_list.push_back(g);
        }
        pending.swap(again_list);
    }
    return join_groups(h);
}

// the group and its local index for replica r, after validating r
int locate(tis_handle *h, int r, Group **g, int *loc)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    if (r < 0 || r >= h->R) return fail(TIS_ERR_ARG, "replica %d out of range (0..%d)", r, h->R - 1);
    *g = h->groups[h->grp_of[r]];
    *loc = h->loc_of[r];
    return TIS_OK;
}

}  // namespace

extern "C" {

int tis_run_params_default(tis_run_params *p)
{
    if (!p) return fail(TIS_ERR_ARG, "null params");
    memset(p, 0, sizeof *p);
    p->precision = TIS_PREC_MIXED;
    p->noise = TIS_NOISE_REFERENCE;
    p->sr = 12.0;
    p->skin = 3.0;
    p->lr_interval = 10;
    p->use_graph = 1;
    p->graph_steps = 20;
    return TIS_OK;
}

int tis_create(const tis_system *const *systems, int n_replicas, const tis_run_params *prm_in, tis_handle **out)
{
    tis::clear_error();
    if (!systems || n_replicas < 1 || !out) return fail(TIS_ERR_ARG, "tis_create: bad argument");
    tis_run_params prm;
    if (prm_in) prm = *prm_in;
    else tis_run_params_default(&prm);
    if (prm.lr_interval < 1) prm.lr_interval = 10;
    if (prm.graph_steps < 1) prm.graph_steps = 20;
    if (prm.sr <= 0) prm.sr = 12.0;
    if (prm.skin <= 0) prm.skin = 3.0;
    if (prm.groups < 0) return fail(TIS_ERR_ARG, "tis_create: negative group count");
    if (prm.fused_ctas < 0 || prm.fused_ctas > 8)
        return fail(TIS_ERR_ARG, "tis_create: fused_ctas %d is not 0 .. 8", prm.fused_ctas);
    if (prm.lanes_sr == 0) prm.lanes_sr = tis::kLanesSR;
    if (prm.lanes_lr == 0) prm.lanes_lr = tis::kLanesLR;
    if (prm.lanes_sr != 1 && prm.lanes_sr != 2 && prm.lanes_sr != 4)
        return fail(TIS_ERR_ARG, "tis_create: lanes_sr %d is not 1, 2 or 4", prm.lanes_sr);
    if (prm.lanes_lr != 2 && prm.lanes_lr != 4 && prm.lanes_lr != 8)
        return fail(TIS_ERR_ARG, "tis_create: lanes_lr %d is not 2, 4 or 8", prm.lanes_lr);
    int G = prm.groups > 0 ? prm.groups : (3 * n_replicas + 15) / 16;  // about 5 1/3 replicas per group
    G = std::min(G, n_replicas);
    prm.groups = G;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(TIS_ERR_CUDA, "no CUDA device available");
    if (prm.device < 0 || prm.device >= ndev) return fail(TIS_ERR_ARG, "device %d out of range", prm.device);
    TIS_CUDA(cudaSetDevice(prm.device));

    tis_handle *h = new tis_handle();
    h->R = n_replicas;
    h->prm = prm;
    auto bail = [&](int rc) {
        delete h;
        return rc;
    };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(TIS_ERR_CUDA, "cudaStreamCreate/cudaEventCreate failed"));
    for (int k = 0; k < G; ++k) {
        // replicas [first, last) in group k: sizes differ by at most one
        const int first = (int)((int64_t)n_replicas * k / G), last = (int)((int64_t)n_replicas * (k + 1) / G);
        Group *g = nullptr;
        const int rc = grp_create(systems + first, last - first, prm, first, &g);
        if (rc) return bail(rc);
        h->groups.push_back(g);
        cudaEvent_t e;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(TIS_ERR_CUDA, "cudaEventCreate failed"));
        h->join.push_back(e);
        for (int r = first; r < last; ++r) {
            h->grp_of.push_back(k);
            h->loc_of.push_back(r - first);
        }
        h->npk += g->npk;
    }
    // one staging buffer for the whole handle: a state upload or read-back is nine
    // copies, whatever the number of groups
    if (cudaMalloc((void **)&h->stage, sizeof(double) * 9 * (size_t)h->npk) != cudaSuccess)
        return bail(fail(TIS_ERR_CUDA, "cudaMalloc of the state staging buffer failed"));
    *out = h;
    return TIS_OK;
}

static void density_release(tis_density *d);

static void ring_free(tis_frame_ring *f);

int tis_destroy(tis_handle *h)
{
    if (h) {
        cudaSetDevice(h->prm.device);
        cudaStreamSynchronize(h->stream);
        if (h->ring) ring_free(h->ring);  // a ring does not outlive its handle
        h->ring = nullptr;
        for (tis_density *d : h->densities) density_release(d);  // the grids stay valid handles, now empty
        h->densities.clear();
        for (Group *g : h->groups) grp_destroy(g);
        h->groups.clear();
        cudaStreamSynchronize(h->stream);
        delete h;
    }
    return TIS_OK;
}

int tis_set_state(tis_handle *h, int r, const double *x, const double *y, const double *z, const double *xo,
                  const double *yo, const double *zo, const double *vx, const double *vy, const double *vz)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_set_state(g, loc, x, y, z, xo, yo, zo, vx, vy, vz);
}

int tis_get_state(tis_handle *h, int r, double *x, double *y, double *z, double *xo, double *yo, double *zo,
                  double *vx, double *vy, double *vz)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_get_state(g, loc, x, y, z, xo, yo, zo, vx, vy, vz);
}

int tis_set_states(tis_handle *h, const double *x, const double *y, const double *z, const double *xo,
                   const double *yo, const double *zo, const double *vx, const double *vy, const double *vz)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    const double *src[9] = {x, y, z, xo, yo, zo, vx, vy, vz};
    for (int c = 0; c < 9; ++c)
        if (!src[c]) return fail(TIS_ERR_ARG, "tis_set_states: null array %d", c);
    const size_t n = (size_t)h->npk;
    for (int c = 0; c < 9; ++c)
        TIS_CUDA(cudaMemcpyAsync(h->stage + c * n, src[c], sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    int64_t off = 0;
    int rc = each_group(h, [&](Group *g) -> int {  // each group unpacks its slice (stride: the handle's npk)
        tis::launch_put_state(g->dev, g->stream, h->stage + off, (int)n);
        off += g->npk;
        g->lists_built = false;
        TIS_CUDA(cudaGetLastError());
        return TIS_OK;
    });
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return TIS_OK;
}

int tis_get_states(tis_handle *h, double *x, double *y, double *z, double *xo, double *yo, double *zo, double *vx,
                   double *vy, double *vz)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    double *dst[9] = {x, y, z, xo, yo, zo, vx, vy, vz};
    unsigned mask = 0;
    for (int c = 0; c < 9; ++c) mask |= dst[c] ? (1u << c) : 0u;
    const size_t n = (size_t)h->npk;
    int64_t off = 0;
    int rc = each_group(h, [&](Group *g) -> int {  // each group packs its slice into the handle's staging buffer
        tis::launch_get_state(g->dev, g->stream, h->stage + off, (int)n, mask);
        off += g->npk;
        TIS_CUDA(cudaGetLastError());
        return TIS_OK;
    });
    if (rc) return rc;
    for (int c = 0; c < 9; ++c)
        if (dst[c]) TIS_CUDA(cudaMemcpyAsync(dst[c], h->stage + c * n, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return TIS_OK;
}

int tis_get_all_energies(tis_handle *h, double *out)
{
    if (!h || !out) return fail(TIS_ERR_ARG, "tis_get_all_energies: bad argument");
    int64_t off = 0;
    int rc = each_group(h, [&](Group *g) {
        const int r = grp_get_all_energies(g, out + 5 * off);
        off += g->R;
        return r;
    });
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return TIS_OK;
}

int tis_populate_lists(tis_handle *h)
{
    Range range("tis_populate_lists");
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    return populate_groups(h, h->groups);
}

int tis_get_cells(tis_handle *h, int r, int32_t *cell, int32_t *dims)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_get_cells(g, loc, cell, dims);
}

int tis_get_pairs(tis_handle *h, int r, int which, int32_t *pairs, int64_t cap, int64_t *n)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_get_pairs(g, loc, which, pairs, cap, n);
}

int tis_ion_counts(tis_handle *h, int r, int kind, double radius, int32_t *counts, int64_t cap, int64_t *n_p,
                   int32_t *total)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_ion_counts(g, loc, kind, radius, counts, cap, n_p, total);
}

}  // extern "C"

struct tis_density {
    tis_handle *h = nullptr;
    Group *g = nullptr;
    int loc = 0, kind = 0, n = 0, n_fit = 0;
    double lo[3] = {0, 0, 0}, delta = 1;
    int dims[3] = {0, 0, 0};
    int *d_idx = nullptr;
    double *d_ref = nullptr, *d_fit = nullptr;
    unsigned long long *d_grid = nullptr;
    int64_t frames = 0;
    size_t cells() const { return (size_t)dims[0] * dims[1] * dims[2]; }
    void release()
    {
        for (void *p : {(void *)d_idx, (void *)d_ref, (void *)d_fit, (void *)d_grid})
            if (p) cudaFree(p);
        d_idx = nullptr;
        d_ref = d_fit = nullptr;
        d_grid = nullptr;
        h = nullptr;
        g = nullptr;
    }
    ~tis_density() { release(); }
};

// the handle is being destroyed: its grids lose their device memory and report
// TIS_ERR_STATE from then on
static void density_release(tis_density *d) { d->release(); }

extern "C" {

int tis_density_create(tis_handle *h, int r, int kind, const double lo[3], double delta, const int32_t dims[3],
                       int32_t n_fit, const int32_t *fit_beads, const double *fit_ref, tis_density **out)
{
    if (!out || !lo || !dims) return fail(TIS_ERR_ARG, "tis_density_create: bad argument");
    *out = nullptr;
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    if (!(delta > 0) || dims[0] < 1 || dims[1] < 1 || dims[2] < 1 ||
        (double)dims[0] * dims[1] * dims[2] > 2147483647.0)
        return fail(TIS_ERR_ARG, "tis_density_create: bad grid (delta %g, dims %d %d %d)", delta, dims[0], dims[1], dims[2]);
    if (kind < 0 || kind > 255) return fail(TIS_ERR_ARG, "tis_density_create: kind %d", kind);
    const RepHost &hr = g->rep[loc];
    if (n_fit < 0 || (n_fit > 0 && (!fit_beads || !fit_ref)) || n_fit == 1 || n_fit == 2)
        return fail(TIS_ERR_ARG, "tis_density_create: a fit needs at least three beads and their reference positions");
    for (int i = 0; i < n_fit; ++i)
        if (fit_beads[i] < 0 || fit_beads[i] >= hr.n) return fail(TIS_ERR_ARG, "tis_density_create: fit bead %d", fit_beads[i]);
    TIS_CUDA(cudaSetDevice(h->prm.device));
    tis_density *d = new tis_density();
    d->h = h;
    d->g = g;
    d->loc = loc;
    d->kind = kind;
    d->n = hr.n;
    d->n_fit = n_fit;
    d->delta = delta;
    for (int a = 0; a < 3; ++a) {
        d->lo[a] = lo[a];
        d->dims[a] = dims[a];
    }
    auto bail = [&](cudaError_t e) {
        delete d;
        return fail(TIS_ERR_NOMEM, "tis_density_create: %s", cudaGetErrorString(e));
    };
    cudaError_t e;
    if ((e = cudaMalloc((void **)&d->d_grid, sizeof(unsigned long long) * d->cells())) != cudaSuccess ||
        (e = cudaMalloc((void **)&d->d_fit, sizeof(double) * 16)) != cudaSuccess ||
        (e = cudaMemset(d->d_grid, 0, sizeof(unsigned long long) * d->cells())) != cudaSuccess ||
        (e = cudaMemset(d->d_fit, 0, sizeof(double) * 16)) != cudaSuccess)
        return bail(e);
    if (n_fit > 0) {
        if ((e = cudaMalloc((void **)&d->d_idx, sizeof(int) * n_fit)) != cudaSuccess ||
            (e = cudaMalloc((void **)&d->d_ref, sizeof(double) * 3 * n_fit)) != cudaSuccess ||
            (e = cudaMemcpy(d->d_idx, fit_beads, sizeof(int) * n_fit, cudaMemcpyHostToDevice)) != cudaSuccess ||
            (e = cudaMemcpy(d->d_ref, fit_ref, sizeof(double) * 3 * n_fit, cudaMemcpyHostToDevice)) != cudaSuccess)
            return bail(e);
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return bail(e);  // memsets and uploads (legacy stream) done
    h->densities.push_back(d);
    *out = d;
    return TIS_OK;
}

int tis_density_add(tis_density *d)
{
    if (!d) return fail(TIS_ERR_ARG, "tis_density_add: null grid");
    if (!d->h) return fail(TIS_ERR_STATE, "tis_density_add: the grid's handle was destroyed");
    TIS_CUDA(cudaSetDevice(d->h->prm.device));
    const tis::Dev &dev = d->g->dev;
    if (d->n_fit > 0) tis::launch_fit(dev, d->h->stream, d->loc, d->n_fit, d->d_idx, d->d_ref, d->d_fit);
    tis::launch_density(dev, d->h->stream, d->loc, d->n, d->kind, d->n_fit > 0 ? d->d_fit : nullptr, d->lo, d->delta,
                        d->dims, d->d_grid);
    TIS_CUDA(cudaGetLastError());
    ++d->frames;
    return TIS_OK;
}

int tis_density_get(tis_density *d, double *counts, int64_t cap, int64_t *frames, double *rmsd)
{
    if (!d) return fail(TIS_ERR_ARG, "tis_density_get: null grid");
    if (!d->h) return fail(TIS_ERR_STATE, "tis_density_get: the grid's handle was destroyed");
    TIS_CUDA(cudaSetDevice(d->h->prm.device));
    std::vector<unsigned long long> c(d->cells());
    double fit[16];
    TIS_CUDA(cudaMemcpyAsync(c.data(), d->d_grid, sizeof(unsigned long long) * c.size(), cudaMemcpyDeviceToHost, d->h->stream));
    TIS_CUDA(cudaMemcpyAsync(fit, d->d_fit, sizeof fit, cudaMemcpyDeviceToHost, d->h->stream));
    TIS_CUDA(cudaStreamSynchronize(d->h->stream));
    if (counts)
        for (size_t i = 0; i < c.size() && (int64_t)i < cap; ++i) counts[i] = (double)c[i];
    if (frames) *frames = d->frames;
    if (rmsd) *rmsd = d->n_fit > 0 ? fit[15] : 0.0;
    return TIS_OK;
}

int tis_density_write_dx(tis_density *d, const char *path)
{
    if (!d || !path) return fail(TIS_ERR_ARG, "tis_density_write_dx: bad argument");
    std::vector<double> c(d->cells());
    int64_t frames = 0;
    int rc = tis_density_get(d, c.data(), (int64_t)c.size(), &frames, nullptr);
    if (rc) return rc;
    FILE *f = fopen(path, "w");
    if (!f) return fail(TIS_ERR_IO, "cannot open %s", path);
    const int *n = d->dims;
    fprintf(f, "# OpenDX grid: ion counts of kind %d accumulated over %lld frames\n", d->kind, (long long)frames);
    fprintf(f, "# bins of %g A; the origin is the centre of bin (0, 0, 0)\n", d->delta);
    fprintf(f, "# values follow the grid positions with the last index (z) varying fastest,\n");
    fprintf(f, "# then y, then x\n");
    fprintf(f, "# written by tis_density_write_dx\n");
    fprintf(f, "# (no comment lines below this one)\n");
    fprintf(f, "object 1 class gridpositions counts %d %d %d\n", n[0], n[1], n[2]);
    fprintf(f, "origin %.6f %.6f %.6f\n", d->lo[0] + 0.5 * d->delta, d->lo[1] + 0.5 * d->delta, d->lo[2] + 0.5 * d->delta);
    fprintf(f, "delta %.6f 0.000000 0.000000\n", d->delta);
    fprintf(f, "delta 0.000000 %.6f 0.000000\n", d->delta);
    fprintf(f, "delta 0.000000 0.000000 %.6f\n", d->delta);
    fprintf(f, "object 2 class gridconnections counts %d %d %d\n", n[0], n[1], n[2]);
    fprintf(f, "object 3 class array type \"double\" rank 0 items %zu data follows\n", c.size());
    for (size_t i = 0; i < c.size(); ++i) fprintf(f, (i % 3 == 2 || i + 1 == c.size()) ? "%.7g\n" : "%.7g ", c[i]);
    fprintf(f, "attribute \"dep\" string \"positions\"\n");
    fprintf(f, "object \"density\" class field\n");
    fprintf(f, "component \"positions\" value 1\n");
    fprintf(f, "component \"connections\" value 2\n");
    fprintf(f, "component \"data\" value 3\n");
    const bool ok = !ferror(f);
    fclose(f);
    return ok ? TIS_OK : fail(TIS_ERR_IO, "short write to %s", path);
}

int tis_density_destroy(tis_density *d)
{
    if (d) {
        if (d->h) {
            cudaSetDevice(d->h->prm.device);
            cudaStreamSynchronize(d->h->stream);
            auto &v = d->h->densities;
            v.erase(std::remove(v.begin(), v.end(), d), v.end());
        }
        delete d;
    }
    return TIS_OK;
}

int tis_get_hb_status(tis_handle *h, int r, int32_t *status, int32_t *excess)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_get_hb_status(g, loc, status, excess);
}

int tis_compute_forces(tis_handle *h, int r, int mask, double *forces, double *energies)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_compute_forces(g, loc, mask, forces, energies);
}

int tis_deterministic_forces(tis_handle *h)
{
    return each_group(h, [](Group *g) { return grp_deterministic_forces(g); });
}

int tis_get_forces(tis_handle *h, int r, double *forces)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_get_forces(g, loc, forces);
}

// Bit-exact checkpoint: every array a step reads and leaves for the next one
// (step_state: x, x_old, v, fixed-point positions, the held LR force, replica
// counters with the rand() position, neighbour lists, H-bond status), per group.
}  // extern "C"

namespace {

// FNV-1a over the replicas' constants that define the simulated system: sizes, box,
// temperature, step, Coulomb strength and screening, cutoffs, centre bead, seeds,
// per-type masses and friction factors, pair tables.  A checkpoint carries it so that
// a handle made from other systems (or seeds) of the same sizes refuses it.
struct Fnv {
    uint64_t h = 1469598103934665603ull;
    template <class T>
    void add(const T *v, size_t n)
    {
        const unsigned char *b = reinterpret_cast<const unsigned char *>(v);
        for (size_t i = 0; i < n * sizeof(T); ++i) h = (h ^ b[i]) * 1099511628211ull;
    }
};

int system_hash(tis_handle *h, uint64_t *out)
{
    Fnv f;
    for (Group *g : h->groups) {
        std::vector<tis::RepParams> rp(g->R);
        TIS_CUDA(cudaMemcpy(rp.data(), g->dev.rp, sizeof(tis::RepParams) * g->R, cudaMemcpyDeviceToHost));
        for (const auto &R : rp) {
            const int ints[6] = {R.n, R.npad, R.nrna, R.center - R.p0, R.lr_interval, R.nc};
            f.add(ints, 6);
            f.add(R.box, 3);
            const double sc[8] = {R.T, R.h, R.lB, R.kappa, R.rc2, R.r2sr, R.r2lr, R.skin};
            f.add(sc, 8);
            f.add(&R.seed, 1);
            f.add(R.mass, 10);
            f.add(R.k1, 10);
            f.add(R.k2, 10);
            f.add(R.sigma, 10);
            f.add(R.dlj2_d, 46);
            f.add(R.flj_d, 46);
            f.add(R.elj_d, 46);
            f.add(R.qclb_d, 46);
        }
    }
    *out = f.h;
    return TIS_OK;
}

struct FileCloser {
    void operator()(FILE *f) const
    {
        if (f) fclose(f);
    }
};
using File = std::unique_ptr<FILE, FileCloser>;

}  // namespace

extern "C" {

// Bit-exact checkpoint, format TISCKPT2: magic, groups and replicas, the system hash,
// then per group its sizes, list capacity, lists-built flag and every step_state array
// (size, bytes).
int tis_checkpoint_save(tis_handle *h, const char *path)
{
    Range range("tis_checkpoint_save");
    if (!h || !path) return fail(TIS_ERR_ARG, "tis_checkpoint_save: bad argument");
    TIS_CUDA(cudaSetDevice(h->prm.device));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    uint64_t hash = 0;
    int rc;
    if ((rc = system_hash(h, &hash))) return rc;
    File f(fopen(path, "wb"));
    if (!f) return fail(TIS_ERR_IO, "cannot open %s", path);
    bool ok = fwrite("TISCKPT2", 1, 8, f.get()) == 8;
    const int32_t head[2] = {(int32_t)h->groups.size(), h->R};
    ok = ok && fwrite(head, 4, 2, f.get()) == 2 && fwrite(&hash, 8, 1, f.get()) == 1;
    std::vector<char> buf;
    for (Group *g : h->groups) {
        if (!ok) break;
        TIS_CUDA(cudaStreamSynchronize(g->stream));
        const int32_t gh[5] = {g->R, g->P, g->dev.cap_sr, g->dev.cap_lr, g->lists_built ? 1 : 0};
        ok = ok && fwrite(gh, 4, 5, f.get()) == 5;
        for (const auto &e : step_state(g)) {
            const uint64_t n = e.second;
            buf.resize(n);
            if (n) TIS_CUDA(cudaMemcpy(buf.data(), e.first, n, cudaMemcpyDeviceToHost));
            ok = ok && fwrite(&n, 8, 1, f.get()) == 1 && fwrite(buf.data(), 1, n, f.get()) == n;
        }
    }
    ok = fclose(f.release()) == 0 && ok;
    return ok ? TIS_OK : fail(TIS_ERR_IO, "short write to %s", path);
}

// The whole file is read and checked against the handle (format, groups, sizes,
// system hash, every array's size) before anything on the device changes; only then
// do the lists take the saved capacity and the arrays their saved contents.
int tis_checkpoint_load(tis_handle *h, const char *path)
{
    Range range("tis_checkpoint_load");
    if (!h || !path) return fail(TIS_ERR_ARG, "tis_checkpoint_load: bad argument");
    TIS_CUDA(cudaSetDevice(h->prm.device));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    File f(fopen(path, "rb"));
    if (!f) return fail(TIS_ERR_IO, "cannot open %s", path);
    auto bad = [&](const char *why) { return fail(TIS_ERR_FORMAT, "%s: %s", path, why); };
    char magic[8];
    int32_t head[2];
    if (fread(magic, 1, 8, f.get()) != 8 || memcmp(magic, "TISCKPT2", 8) != 0 || fread(head, 4, 2, f.get()) != 2)
        return bad("not a checkpoint written by tis_checkpoint_save");
    if (head[0] != (int32_t)h->groups.size() || head[1] != h->R)
        return bad("replica groups or replicas differ from the handle's");
    uint64_t saved = 0, mine = 0;
    int rc;
    if (fread(&saved, 8, 1, f.get()) != 1) return bad("truncated");
    if ((rc = system_hash(h, &mine))) return rc;
    if (saved != mine) return bad("written for other systems, parameters or seeds than the handle's");
    struct GroupData {
        int32_t gh[5];
        std::vector<std::vector<char>> arrays;
    };
    std::vector<GroupData> data(h->groups.size());
    for (size_t gi = 0; gi < h->groups.size(); ++gi) {
        Group *g = h->groups[gi];
        GroupData &D = data[gi];
        if (fread(D.gh, 4, 5, f.get()) != 5) return bad("truncated");
        if (D.gh[0] != g->R || D.gh[1] != g->P) return bad("a replica group's size differs from the handle's");
        if (D.gh[2] < 1 || D.gh[3] < 1) return bad("bad list capacity");
        // step_state's sizes at the saved list capacity (the lists are its last two arrays)
        std::vector<std::pair<void *, size_t>> want = step_state(g);
        for (auto &e : want) {
            if (e.first == (void *)g->dev.nbr_sr) e.second = sizeof(int) * (size_t)D.gh[2] * g->P;
            if (e.first == (void *)g->dev.nbr_lr) e.second = sizeof(int) * (size_t)D.gh[3] * g->P;
        }
        for (const auto &e : want) {
            uint64_t n = 0;
            if (fread(&n, 8, 1, f.get()) != 1 || n != e.second) return bad("an array's size differs from the handle's");
            D.arrays.emplace_back(n);
            if (n && fread(D.arrays.back().data(), 1, n, f.get()) != n) return bad("truncated");
        }
    }
    if (fgetc(f.get()) != EOF) return bad("trailing bytes after the last group");
    f.reset();
    for (size_t gi = 0; gi < h->groups.size(); ++gi) {
        Group *g = h->groups[gi];
        const GroupData &D = data[gi];
        TIS_CUDA(cudaStreamSynchronize(g->stream));
        if (D.gh[2] != g->dev.cap_sr || D.gh[3] != g->dev.cap_lr) {
            if ((rc = grow_lists(g, D.gh[2], D.gh[3]))) return rc;  // the saved list capacity
        }
        const auto st = step_state(g);
        for (size_t k = 0; k < st.size(); ++k)
            if (st[k].second) TIS_CUDA(cudaMemcpy(st[k].first, D.arrays[k].data(), st[k].second, cudaMemcpyHostToDevice));
        g->lists_built = D.gh[4] != 0;
    }
    // pageable uploads may still be in flight when cudaMemcpy returns; the next
    // step runs on non-blocking streams
    TIS_CUDA(cudaDeviceSynchronize());
    return TIS_OK;
}

int tis_param_grad(tis_handle *h, double *out)
{
    Range range("tis_param_grad");
    if (!h || !out) return fail(TIS_ERR_ARG, "tis_param_grad: bad argument");
    return each_group(h, [&](Group *g) { return grp_param_grad(g, out + (size_t)g->base * tis::kNParams); });
}

int tis_traj_grad(tis_handle *h, int64_t steps, int32_t checkpoint_every, const double *const *seed, double *dtheta,
                  double *const *dstate0)
{
    Range range("tis_traj_grad");
    if (!h || steps < 1 || checkpoint_every < 1 || !dtheta) return fail(TIS_ERR_ARG, "tis_traj_grad: bad argument");
    int64_t off = 0;
    return each_group(h, [&](Group *g) {
        const int rc = grp_traj_grad(g, steps, checkpoint_every, seed, off, dtheta + (size_t)g->base * tis::kNParams, dstate0);
        off += g->npk;
        return rc;
    });
}

int tis_full_forces(tis_handle *h)
{
    return each_group(h, [](Group *g) { return grp_full_forces(g); });
}

int tis_move_rigid_units(tis_handle *h)
{
    return each_group(h, [](Group *g) { return grp_move_rigid_units(g); });
}

int tis_check_shifts(tis_handle *h)
{
    return each_group(h, [](Group *g) { return grp_check_shifts(g); });
}

}  // extern "C"

namespace {

// `steps` steps of the group as launches of the persistent fused step kernel (at
// most kFusedChunk steps per launch)
constexpr int kFusedChunk = 1000;
int enqueue_fused(Group *g, int64_t steps, int ctas)
{
    for (int64_t done = 0; done < steps;) {
        const int n = (int)std::min<int64_t>(kFusedChunk, steps - done);
        const int e = tis::launch_step_fused(g->dev, g->stream, n, ctas);
        if (e != 0) return fail(TIS_ERR_CUDA, "fused step kernel launch: %s", cudaGetErrorString((cudaError_t)e));
        done += n;
    }
    return TIS_OK;
}

// `steps` fused steps of every group captured from the handle's stream into one
// graph: the fork, each group's steps on its own streams, the join
int capture_handle(tis_handle *h, int steps, tis_handle::StepGraph *sg)
{
    // no graph of the handle is in flight while one is replaced, captured,
    // instantiated and uploaded
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    if (sg->exec) cudaGraphExecDestroy(sg->exec);
    sg->exec = nullptr;
    sg->steps = 0;
    TIS_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = fork_groups(h);
    for (Group *g : h->groups) {
        if (rc) break;
        if (h->prm.fused_ctas > 0) rc = enqueue_fused(g, steps, h->prm.fused_ctas);
        else
            for (int s = 0; s < steps; ++s) enqueue_step(g);
    }
    if (rc == TIS_OK) rc = join_groups(h);
    cudaGraph_t gr = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->stream, &gr);
    if (rc) {
        if (gr) cudaGraphDestroy(gr);
        return rc;
    }
    if (e != cudaSuccess) return fail(TIS_ERR_CUDA, "capture of the step graph: %s", cudaGetErrorString(e));
    const cudaError_t ei = cudaGraphInstantiate(&sg->exec, gr, 0);
    cudaGraphDestroy(gr);
    if (ei != cudaSuccess) return fail(TIS_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(ei));
    // the graph's work moved to the device now, not at its first launch
    TIS_CUDA(cudaGraphUpload(sg->exec, h->stream));
    sg->steps = steps;
    sg->gens.clear();
    for (Group *g : h->groups) sg->gens.push_back(g->list_gen);
    return TIS_OK;
}

// list builds of the groups whose lists are not built, ordered after the work
// queued on the handle's stream
int build_missing_lists(tis_handle *h)
{
    std::vector<Group *> need;
    for (Group *g : h->groups)
        if (!g->lists_built) need.push_back(g);
    return need.empty() ? TIS_OK : populate_groups(h, need);
}

// the handle's graph of `steps` steps in slot sg, captured again when its length
// differs or a group's lists moved since its capture
int handle_graph(tis_handle *h, int steps, tis_handle::StepGraph *sg)
{
    bool fresh = sg->exec && sg->steps == steps && sg->gens.size() == h->groups.size();
    for (size_t k = 0; fresh && k < h->groups.size(); ++k) fresh = sg->gens[k] == h->groups[k]->list_gen;
    return fresh ? TIS_OK : capture_handle(h, steps, sg);
}

}  // namespace

extern "C" {

// n fused steps of every replica.  With use_graph, from CUDA graphs of the whole
// handle (one launch for all groups): the graph_steps-long graph replayed
// n / graph_steps times, then a graph of the remaining steps (kept for the next
// call with the same remainder); else direct launches.
int tis_step(tis_handle *h, int64_t n)
{
    Range range("tis_step");
    if (!h || n < 0) return fail(TIS_ERR_ARG, "tis_step: bad argument");
    int rc;
    if (n == 0) return TIS_OK;
    if (h->prm.fused_ctas > 0 && !h->prm.use_graph) {
        if ((rc = build_missing_lists(h))) return rc;
        const int ctas = h->prm.fused_ctas;
        rc = each_group(h, [n, ctas](Group *g) { return enqueue_fused(g, n, ctas); });
        if (rc) return rc;
        for (Group *g : h->groups) g->launches += (n + kFusedChunk - 1) / kFusedChunk;
        return TIS_OK;
    }
    if (!h->prm.use_graph) return each_group(h, [n](Group *g) { return grp_step(g, n); });
    if ((rc = build_missing_lists(h))) return rc;
    const int gs = std::max(1, (int)h->prm.graph_steps);
    const int64_t full = n / gs, rem = n % gs;
    if (full > 0) {
        if ((rc = handle_graph(h, gs, &h->full))) return rc;
        for (int64_t k = 0; k < full; ++k) TIS_CUDA(cudaGraphLaunch(h->full.exec, h->stream));
    }
    if (rem > 0) {
        if ((rc = handle_graph(h, (int)rem, &h->tail))) return rc;
        TIS_CUDA(cudaGraphLaunch(h->tail.exec, h->stream));
    }
    for (Group *g : h->groups)  // kernel launches: per step, or per graph of the fused kernel
        g->launches += h->prm.fused_ctas > 0 ? full * ((gs + kFusedChunk - 1) / kFusedChunk) + (rem > 0 ? 1 : 0)
                                             : n * tis::kernel_launches_per_step();
    return TIS_OK;
}

int tis_capture_graph(tis_handle *h, int32_t steps)
{
    if (!h || steps < 1) return fail(TIS_ERR_ARG, "tis_capture_graph: bad argument");
    h->prm.graph_steps = steps;
    h->prm.use_graph = 1;
    for (Group *g : h->groups) {
        g->prm.graph_steps = steps;
        g->prm.use_graph = 1;
    }
    int rc;
    if ((rc = build_missing_lists(h))) return rc;
    return capture_handle(h, steps, &h->full);
}

int tis_profile_stages(tis_handle *h, int64_t n, double *ms)
{
    // stage times of the groups run one after another, summed over the groups
    if (!h || n < 1 || !ms) return fail(TIS_ERR_ARG, "tis_profile_stages: bad argument");
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < TIS_N_STAGES; ++k) ms[k] = 0;
    for (Group *g : h->groups) {
        double part[TIS_N_STAGES];
        const int rc = grp_profile_stages(g, n, part);
        if (rc) return rc;
        for (int k = 0; k < TIS_N_STAGES; ++k) ms[k] += part[k];
    }
    return TIS_OK;
}

// Every stage's kernel timed inside the concurrently replayed step graphs of all
// groups: each group's `steps` steps captured once more with an event pair around
// each of the eight kernels of every step, the groups' graphs forked from the
// handle's stream and replayed together, the event pairs' durations averaged over
// steps and groups.  Advances every replica by `steps` steps like tis_step.
int tis_profile_in_step(tis_handle *h, int32_t steps, double *ms)
{
    if (!h || steps < 1 || steps > 1000 || !ms) return fail(TIS_ERR_ARG, "tis_profile_in_step: bad argument");
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    const size_t n_ev = 2 * (size_t)steps * TIS_N_STAGES;
    const size_t G = h->groups.size();
    std::vector<cudaEvent_t> ev(n_ev * G, nullptr);
    std::vector<cudaGraphExec_t> exec(G, nullptr);
    int rc = TIS_OK;
    auto cleanup = [&]() {
        for (auto e : exec)
            if (e) cudaGraphExecDestroy(e);
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
        for (Group *g : h->groups) {
            g->pev = nullptr;
            g->pev_next = 0;
        }
    };
    for (auto &e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) {
            cleanup();
            return fail(TIS_ERR_CUDA, "tis_profile_in_step: cudaEventCreate failed");
        }
    for (size_t gi = 0; gi < G && !rc; ++gi) {
        Group *g = h->groups[gi];
        if (!g->lists_built && (rc = populate(g))) break;
        g->pev = &ev[gi * n_ev];
        g->pev_next = 0;
        rc = capture_steps(g, steps, &exec[gi]);
        g->pev = nullptr;
    }
    if (!rc) rc = fork_groups(h);
    for (size_t gi = 0; gi < G && !rc; ++gi)
        if (cudaGraphLaunch(exec[gi], h->groups[gi]->stream) != cudaSuccess)
            rc = fail(TIS_ERR_CUDA, "tis_profile_in_step: cudaGraphLaunch failed");
    if (!rc) rc = join_groups(h);
    if (!rc && cudaStreamSynchronize(h->stream) != cudaSuccess)
        rc = fail(TIS_ERR_CUDA, "tis_profile_in_step: %s", cudaGetErrorString(cudaGetLastError()));
    if (!rc) {
        for (int k = 0; k < TIS_N_STAGES && !rc; ++k) {
            double acc = 0;
            for (size_t gi = 0; gi < G && !rc; ++gi)
                for (int st = 0; st < steps; ++st) {
                    float t = 0;
                    const size_t b = gi * n_ev + 2 * ((size_t)st * TIS_N_STAGES + k);
                    const cudaError_t e = cudaEventElapsedTime(&t, ev[b], ev[b + 1]);
                    if (e != cudaSuccess) {
                        rc = fail(TIS_ERR_CUDA, "tis_profile_in_step: cudaEventElapsedTime: %s", cudaGetErrorString(e));
                        break;
                    }
                    acc += t;
                }
            ms[k] = acc / ((double)steps * G);
        }
        for (Group *g : h->groups) g->launches += (long long)steps * tis::kernel_launches_per_step();
    }
    cleanup();
    if (rc) return rc;
    for (Group *g : h->groups)
        if ((rc = check_flags(g))) return rc;
    return TIS_OK;
}

// The persistent fused step kernel run for `steps` steps with its phase timer on:
// out[0..5] the mean microseconds per step of its phases (forces, of them the H-bond
// chain, shift, move, control, and the rebuild per step that rebuilds), out[6] the
// share of steps with an LR refresh, out[7] rebuilds per step, out[8..11] the H-bond
// chain's restraint terms, Monte Carlo, forces and Gaussians; means over replicas.
int tis_profile_fused(tis_handle *h, int32_t steps, int32_t ctas, double *out)
{
    if (!h || steps < 1 || ctas < 1 || ctas > 8 || !out) return fail(TIS_ERR_ARG, "tis_profile_fused: bad argument");
    int rc;
    if ((rc = build_missing_lists(h))) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    std::vector<double> acc(tis::kFusedPhases, 0.0);
    for (Group *g : h->groups) {
        unsigned long long *buf = nullptr;
        const size_t n = (size_t)g->R * tis::kFusedPhases;
        TIS_CUDA(cudaMalloc(&buf, n * sizeof(unsigned long long)));
        cudaMemsetAsync(buf, 0, n * sizeof(unsigned long long), g->stream);
        g->dev.fprof = buf;
        const int e = tis::launch_step_fused(g->dev, g->stream, steps, ctas);
        g->dev.fprof = nullptr;
        std::vector<unsigned long long> hb(n);
        cudaError_t ce = e ? (cudaError_t)e : cudaStreamSynchronize(g->stream);
        if (ce == cudaSuccess) ce = cudaMemcpy(hb.data(), buf, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
        cudaFree(buf);
        if (ce != cudaSuccess) return fail(TIS_ERR_CUDA, "tis_profile_fused: %s", cudaGetErrorString(ce));
        for (int r = 0; r < g->R; ++r)
            for (int k = 0; k < tis::kFusedPhases; ++k) acc[k] += (double)hb[(size_t)r * tis::kFusedPhases + k];
        g->launches += 1;
        if ((rc = check_flags(g))) return rc;
    }
    const double reps = (double)h->R, st = (double)steps;
    for (int k = 0; k < 5; ++k) out[k] = acc[k] / reps / st * 1e-3;
    out[5] = acc[7] > 0 ? acc[5] / acc[7] * 1e-3 : 0.0;
    out[6] = acc[6] / reps / st;
    out[7] = acc[7] / reps / st;
    for (int k = 8; k < 12; ++k) out[k] = acc[k] / reps / st * 1e-3;
    return TIS_OK;
}

}  // extern "C"

// The frame ring: pinned, device-mapped host memory the step's kernels write frames
// into (layout in tis::FrameRing), and what the host needs to read it back.
struct tis_frame_ring {
    tis_handle *h = nullptr;
    int every = 0, depth = 0, R = 0;
    int64_t n = 0;
    double *pos = nullptr, *en = nullptr;
    long long *done = nullptr;
};

static void ring_free(tis_frame_ring *f)
{
    if (!f) return;
    if (f->pos) cudaFreeHost(f->pos);
    if (f->en) cudaFreeHost(f->en);
    if (f->done) cudaFreeHost(f->done);
    delete f;
}

namespace {

// the ring's device view in every group (NULL detaches); the step graphs hold the
// kernels' arguments, so they are captured again
int ring_attach(tis_handle *h, const tis_frame_ring *f)
{
    int64_t pk_base = 0;
    for (Group *g : h->groups) {
        tis::FrameRing fr{};
        if (f) {
            TIS_CUDA(cudaHostGetDevicePointer((void **)&fr.pos, f->pos, 0));
            TIS_CUDA(cudaHostGetDevicePointer((void **)&fr.en, f->en, 0));
            TIS_CUDA(cudaHostGetDevicePointer((void **)&fr.done, f->done, 0));
            fr.n_total = f->n;
            fr.pk_base = pk_base;
            fr.R_total = f->R;
            fr.rep_base = g->base;
            fr.every = f->every;
            fr.depth = f->depth;
        }
        g->dev.fr = fr;
        drop_graphs(g);
        pk_base += g->npk;
    }
    return TIS_OK;
}

}  // namespace

extern "C" {

int tis_frames_start(tis_handle *h, int32_t every, int32_t depth, tis_frame_ring **out)
{
    if (!h || every < 1 || depth < 2 || !out) return fail(TIS_ERR_ARG, "tis_frames_start: bad argument");
    if (h->ring) return fail(TIS_ERR_STATE, "tis_frames_start: the handle already writes frames");
    TIS_CUDA(cudaSetDevice(h->prm.device));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    auto *f = new tis_frame_ring;
    f->h = h;
    f->every = every;
    f->depth = depth;
    f->R = h->R;
    for (Group *g : h->groups) f->n += g->npk;
    const unsigned fl = cudaHostAllocMapped | cudaHostAllocPortable;
    cudaError_t e = cudaHostAlloc((void **)&f->pos, sizeof(double) * 3 * (size_t)f->n * depth, fl);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&f->en, sizeof(double) * 5 * (size_t)f->R * depth, fl);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&f->done, sizeof(long long) * (size_t)f->R * depth, fl);
    if (e != cudaSuccess) {
        ring_free(f);
        return fail(TIS_ERR_CUDA, "tis_frames_start: pinned host memory: %s", cudaGetErrorString(e));
    }
    for (size_t k = 0; k < (size_t)f->R * depth; ++k) f->done[k] = -1;
    const int rc = ring_attach(h, f);
    if (rc) {
        ring_attach(h, nullptr);
        ring_free(f);
        return rc;
    }
    h->ring = f;
    *out = f;
    return TIS_OK;
}

int tis_frames_read(tis_frame_ring *f, int64_t klok, double *x, double *y, double *z, double *energies)
{
    if (!f || !f->h) return fail(TIS_ERR_ARG, "tis_frames_read: null ring");
    if (klok < f->every || klok % f->every != 0)
        return fail(TIS_ERR_ARG, "tis_frames_read: step %lld is not a frame step (every %d)", (long long)klok, f->every);
    const size_t slot = (size_t)((klok / f->every) % f->depth);
    const volatile long long *done = f->done + slot * f->R;
    auto state = [&](bool *ready, bool *gone) {
        *ready = true;
        *gone = false;
        for (int r = 0; r < f->R; ++r) {
            const long long v = done[r];
            *ready = *ready && v == klok;
            *gone = *gone || v > klok;
        }
    };
    bool ready, gone;
    state(&ready, &gone);
    if (!ready && !gone) {  // not written yet: wait for the work queued so far
        TIS_CUDA(cudaStreamSynchronize(f->h->stream));
        state(&ready, &gone);
    }
    if (gone) return fail(TIS_ERR_STATE, "tis_frames_read: the frame of step %lld was overwritten", (long long)klok);
    if (!ready) return fail(TIS_ERR_STATE, "tis_frames_read: no frame of step %lld was written", (long long)klok);
    const size_t n = (size_t)f->n;
    const double *p = f->pos + slot * 3 * n;
    if (x) memcpy(x, p, sizeof(double) * n);
    if (y) memcpy(y, p + n, sizeof(double) * n);
    if (z) memcpy(z, p + 2 * n, sizeof(double) * n);
    if (energies) memcpy(energies, f->en + slot * 5 * (size_t)f->R, sizeof(double) * 5 * f->R);
    state(&ready, &gone);  // still the same frame after the copy
    if (!ready) return fail(TIS_ERR_STATE, "tis_frames_read: the frame of step %lld was overwritten while read", (long long)klok);
    return TIS_OK;
}

int tis_frames_stop(tis_frame_ring *f)
{
    if (!f || !f->h) return fail(TIS_ERR_ARG, "tis_frames_stop: null ring");
    tis_handle *h = f->h;
    TIS_CUDA(cudaSetDevice(h->prm.device));
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    ring_attach(h, nullptr);
    h->ring = nullptr;
    ring_free(f);
    return TIS_OK;
}

int tis_sync(tis_handle *h)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    for (Group *g : h->groups) {
        const int rc = grp_sync(g);
        if (rc) return rc;
    }
    return TIS_OK;
}

int tis_get_energies(tis_handle *h, int r, double *out5)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_get_energies(g, loc, out5);
}

int tis_get_stack_energies(tis_handle *h, int r, double *out, int64_t cap, int64_t *n)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_get_stack_energies(g, loc, out, cap, n);
}

int tis_get_counters(tis_handle *h, int r, int64_t *klok, int64_t *rebuilds, int64_t *draws)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    TIS_CUDA(cudaStreamSynchronize(h->stream));
    return grp_get_counters(g, loc, klok, rebuilds, draws);
}

int tis_get_info(tis_handle *h, int *n_replicas, int *device, void **stream)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    if (n_replicas) *n_replicas = h->R;
    if (device) *device = h->prm.device;
    if (stream) *stream = (void *)h->stream;
    return TIS_OK;
}

int tis_replica_size(tis_handle *h, int r, int *n_particles)
{
    Group *g;
    int loc, rc = locate(h, r, &g, &loc);
    if (rc) return rc;
    return grp_replica_size(g, loc, n_particles);
}

int tis_get_launch_count(tis_handle *h, int64_t *n)
{
    if (!h || !n) return fail(TIS_ERR_ARG, "bad argument");
    int64_t total = 0;
    for (Group *g : h->groups) total += g->launches;
    *n = total;
    return TIS_OK;
}

}  // extern "C"
