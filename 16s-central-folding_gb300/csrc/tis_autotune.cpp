// tis_autotune: the launch configuration chosen by measurement (no counterpart in
// the reference, whose loops have no launch shape).  The knobs are the replica
// groups (how many groups' step chains run concurrently), the steps per captured
// graph, the threads per particle of the SR and LR pair launches, and whether the
// steps run in the persistent fused step kernel (with 1, 2 or 4 CTAs per replica)
// instead of the chain of separate kernels; each is tuned in turn
// with the others held (coordinate descent), every trial a fresh handle timed with
// CUDA events on its stream after a warm-up that includes the graph captures.  The
// configuration is tuned for calls of `steps` steps: a trial times as many such
// calls as make up at least kTrialSteps steps, so that a caller stepping a few steps
// per call (one graph launch each) gets the shape that is fastest for that.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "tis_host.h"

using tis::fail;

namespace {

constexpr int64_t kTrialSteps = 1000;  // steps timed per trial at least

double scalar(const tis_system *s, const char *name, double def)
{
    int dt = 0;
    const void *p = nullptr;
    int64_t n = 0;
    if (tis_system_get(s, name, &dt, &p, &n) != TIS_OK || n < 1 || !p) return def;
    if (dt == TIS_F64) return ((const double *)p)[0];
    if (dt == TIS_I64) return (double)((const int64_t *)p)[0];
    return (double)((const int32_t *)p)[0];
}

// the workload's key in the cache file
std::string key_of(const tis_system *const *systems, int n, const tis_run_params &p, int64_t steps)
{
    double particles = 0;
    for (int r = 0; r < n; ++r) particles += scalar(systems[r], "n_particles", 0);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, p.device);
    std::string dev = prop.name;
    for (char &c : dev)
        if (c == ' ') c = '_';
    char buf[512];
    snprintf(buf, sizeof buf, "replicas=%d particles=%.0f box=%.3f rc=%.3f precision=%d noise=%d sr=%.3f skin=%.3f "
                              "lr_interval=%d full_lists=%d steps_per_call=%lld device=%s",
             n, particles, scalar(systems[0], "box", 0), scalar(systems[0], "rc", 0), p.precision, p.noise, p.sr,
             p.skin, p.lr_interval, p.full_lists, (long long)steps, dev.c_str());
    return buf;
}

bool cache_lookup(const char *path, const std::string &key, tis_run_params *p, double *rate)
{
    FILE *f = fopen(path, "r");
    if (!f) return false;
    char line[1024];
    bool found = false;
    while (fgets(line, sizeof line, f)) {
        const char *bar = strstr(line, " | ");
        if (!bar || std::string(line, bar - line) != key) continue;
        int g, gs, ls, ll, fc;
        double r;
        if (sscanf(bar + 3, "groups=%d graph_steps=%d lanes_sr=%d lanes_lr=%d fused_ctas=%d rate=%lf", &g, &gs, &ls, &ll,
                   &fc, &r) == 6) {
            p->groups = g;
            p->graph_steps = gs;
            p->lanes_sr = ls;
            p->lanes_lr = ll;
            p->fused_ctas = fc;
            if (rate) *rate = r;
            found = true;  // the last line for the key wins
        }
    }
    fclose(f);
    return found;
}

// replica-steps/s of one configuration in calls of `steps` steps, or a negative
// value if it failed
double measure(const tis_system *const *systems, int n, const tis_run_params &p, int64_t steps)
{
    tis_handle *h = nullptr;
    if (tis_create(systems, n, &p, &h) != TIS_OK) return -1;
    double rate = -1;
    void *sp = nullptr;
    int nr = 0, dev = 0;
    cudaEvent_t a = nullptr, b = nullptr;
    const int64_t calls = std::max<int64_t>(1, (kTrialSteps + steps - 1) / steps);
    // the warm-up captures the graphs the timed calls replay (a call's remainder too)
    if (tis_get_info(h, &nr, &dev, &sp) == TIS_OK && tis_populate_lists(h) == TIS_OK &&
        tis_step(h, p.graph_steps + 10) == TIS_OK && (steps % p.graph_steps == 0 || tis_step(h, steps) == TIS_OK) &&
        tis_sync(h) == TIS_OK && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess) {
        cudaStream_t s = (cudaStream_t)sp;
        cudaEventRecord(a, s);
        int rc = TIS_OK;
        for (int64_t c = 0; c < calls && rc == TIS_OK; ++c) rc = tis_step(h, steps);
        cudaEventRecord(b, s);
        float ms = 0;
        if (rc == TIS_OK && tis_sync(h) == TIS_OK && cudaEventSynchronize(b) == cudaSuccess &&
            cudaEventElapsedTime(&ms, a, b) == cudaSuccess && ms > 0)
            rate = (double)n * (double)(steps * calls) / (ms * 1e-3);
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    tis_destroy(h);
    return rate;
}

}  // namespace

extern "C" int tis_autotune(const tis_system *const *systems, int n_replicas, const tis_run_params *base, int64_t steps,
                            const char *cache, tis_run_params *best, double *rate)
{
    if (!systems || n_replicas < 1 || !best) return fail(TIS_ERR_ARG, "tis_autotune: bad argument");
    tis_run_params p;
    if (base) p = *base;
    else tis_run_params_default(&p);
    if (steps <= 0) steps = 300;
    p.use_graph = 1;
    if (p.graph_steps < 1) p.graph_steps = 100;
    if (p.groups <= 0) p.groups = std::min(n_replicas, (3 * n_replicas + 15) / 16);
    if (p.lanes_sr == 0) p.lanes_sr = 1;
    if (p.lanes_lr == 0) p.lanes_lr = 4;
    const std::string key = key_of(systems, n_replicas, p, steps);
    if (cache && cache_lookup(cache, key, &p, rate)) {
        *best = p;
        return TIS_OK;
    }
    double cur = measure(systems, n_replicas, p, steps);
    if (cur < 0) {
        char buf[512];
        tis_last_error(buf, sizeof buf);
        return fail(TIS_ERR_CUDA, "tis_autotune: the starting configuration failed: %s", buf);
    }
    auto tune = [&](int32_t tis_run_params::*field, std::vector<int> values) {
        std::sort(values.begin(), values.end());
        values.erase(std::unique(values.begin(), values.end()), values.end());
        for (int v : values) {
            if (v == p.*field) continue;
            tis_run_params q = p;
            q.*field = v;
            const double r = measure(systems, n_replicas, q, steps);
            if (r > cur) {
                cur = r;
                p = q;
            }
        }
    };
    std::vector<int> groups;
    for (int g : {1, 2, n_replicas / 16, n_replicas / 8, n_replicas / 6, (3 * n_replicas + 15) / 16, n_replicas / 4,
                  n_replicas / 3, n_replicas / 2})
        if (g >= 1 && g <= n_replicas) groups.push_back(g);
    tune(&tis_run_params::groups, groups);
    tune(&tis_run_params::graph_steps, {25, 50, 100, 200});
    tune(&tis_run_params::lanes_sr, {1, 2, 4});
    tune(&tis_run_params::lanes_lr, {2, 4, 8});
    tune(&tis_run_params::groups, groups);  // again: the best grouping moves with the launch shapes
    tune(&tis_run_params::fused_ctas, {0, 1, 2, 4});
    *best = p;
    if (rate) *rate = cur;
    if (cache) {
        FILE *f = fopen(cache, "a");
        if (f) {
            fprintf(f, "%s | groups=%d graph_steps=%d lanes_sr=%d lanes_lr=%d fused_ctas=%d rate=%.1f\n", key.c_str(),
                    p.groups, p.graph_steps, p.lanes_sr, p.lanes_lr, p.fused_ctas, cur);
            fclose(f);
        }
    }
    tis::clear_error();
    return TIS_OK;
}
