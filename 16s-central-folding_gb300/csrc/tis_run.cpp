// tis_run: the reference program's command line and output on the GPU engine.
//
//   tis_run [-D<ss_D>] [-E<hs_D>] [-d<st_D>] [-T<T>] [-c<c_Mg>] [-f<c_K>] [-s<seed>]
//           [--steps N] [--every N] [--replicas R] [--precision mixed|fp64] [--device K]
//           [--pdb F] [--bonds F] [--stacks F] [--maxikey F] [--box L] [--rc A] [--center B]
//           [--checkpoint FILE] [--dcd] [--tune] [--debye A]
//
// The single-letter flags are the reference's (E:6082-6099) with its defaults;
// the input files default to the reference's names in the working directory.
// Output: the reference's Contacts, Coordinates and Energies files, named as it
// names them (E:6113-6117), one frame every --every steps (10^6), snapshot copies
// every 5 * 10^6 steps with the copy three snapshots back removed (E:6314-6372),
// and its restart: an existing Coordinates file resumes from its last frame, at
// step frames * every, with x_old = x - v h (E:6181-6211).  --replicas R runs seeds s, s+1, ..., s+R-1 in
// one process, each with its own files.  Steps run to --steps (default the
// reference's 3 * 10^9).  Beyond the reference: --checkpoint FILE saves the whole
// engine state at every frame and, when FILE exists at start, continues from it
// bit for bit instead of the positions-only restart; --dcd also appends every frame
// to a DCD trajectory per replica (Trajectory_..._s<seed>.dcd); --tune measures the
// launch configuration first (cached in tis_tune.txt); --debye A screens the
// Coulomb term as q_i q_j lB exp(-r / A) / r (0, the default: the reference's plain
// truncated Coulomb).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tis_gpu.h"

namespace {

int report(int rc, const char *what)
{
    if (rc) {
        char buf[512];
        tis_last_error(buf, sizeof buf);
        fprintf(stderr, "tis_run: %s: error %d: %s\n", what, rc, buf);
    }
    return rc;
}

bool copy_file(const std::string &from, const std::string &to)
{
    FILE *a = fopen(from.c_str(), "rb");
    if (!a) return false;
    FILE *b = fopen(to.c_str(), "wb");
    if (!b) {
        fclose(a);
        return false;
    }
    std::vector<char> buf(1 << 20);
    size_t n;
    bool ok = true;
    while ((n = fread(buf.data(), 1, buf.size(), a)) > 0) ok = ok && fwrite(buf.data(), 1, n, b) == n;
    fclose(a);
    fclose(b);
    return ok;
}

struct Names {
    std::string contacts, coordinates, energies;
};

// E:6113-6117: Contacts_16SCD_EPS_Mg_Cl_K_D%.3f_E%.3f_d%.3f_T%.3f_cM%.4f_f%.3f_s%d.dat
// (snapshot: the snapshot copy's name, E:6320, with _<index> before .dat)
Names names(const tis_load_params &lp, int seed, bool snapshot = false, long long snap = 0)
{
    char tail[256];
    if (snapshot)
        snprintf(tail, sizeof tail, "D%.3f_E%.3f_d%.3f_T%.3f_cM%.4f_f%.3f_s%d_%lld.dat", lp.ss_D, lp.hs_D, lp.st_D, lp.T,
                 lp.c_mg, lp.c_k, seed, snap);
    else
        snprintf(tail, sizeof tail, "D%.3f_E%.3f_d%.3f_T%.3f_cM%.4f_f%.3f_s%d.dat", lp.ss_D, lp.hs_D, lp.st_D, lp.T,
                 lp.c_mg, lp.c_k, seed);
    return {std::string("Contacts_16SCD_EPS_Mg_Cl_K_") + tail, std::string("Coordinates_16SCD_EPS_Mg_Cl_K_") + tail,
            std::string("Energies_16SCD_EPS_Mg_Cl_K_") + tail};
}

}  // namespace

int main(int argc, char **argv)
{
    tis_load_params lp;
    tis_load_params_default(&lp);
    lp.pdb = "16SCD.pdb";
    lp.bonds = "16SCD_16SCD_unprocessed_bonds.dat";
    lp.stacks = "16SCD_16SCD_unprocessed_stacks.dat";
    lp.maxikey = "MAXIKEY_Mg_Cl_K.dat";
    tis_run_params rp;
    tis_run_params_default(&rp);
    long long steps = 3000000000LL, every = 1000000, snap_every = 5000000;
    int replicas = 1;
    std::string ckpt;
    bool dcd = false, tune = false;
    double debye = 0.0;  // Debye length of a screened Coulomb term (0: the reference's plain Coulomb)
    for (int i = 1; i < argc; ++i) {
        const char *a = argv[i];
        auto next = [&](const char *flag) -> const char * {
            if (i + 1 >= argc) {
                fprintf(stderr, "tis_run: %s needs a value\n", flag);
                exit(2);
            }
            return argv[++i];
        };
        if (!strcmp(a, "--steps")) steps = atoll(next(a));
        else if (!strcmp(a, "--every")) every = atoll(next(a));
        else if (!strcmp(a, "--snapshot-every")) snap_every = atoll(next(a));
        else if (!strcmp(a, "--replicas")) replicas = atoi(next(a));
        else if (!strcmp(a, "--device")) rp.device = atoi(next(a));
        else if (!strcmp(a, "--precision")) rp.precision = strcmp(next(a), "fp64") ? TIS_PREC_MIXED : TIS_PREC_FP64;
        else if (!strcmp(a, "--pdb")) lp.pdb = next(a);
        else if (!strcmp(a, "--bonds")) lp.bonds = next(a);
        else if (!strcmp(a, "--stacks")) lp.stacks = next(a);
        else if (!strcmp(a, "--maxikey")) lp.maxikey = next(a);
        else if (!strcmp(a, "--box")) lp.box = atof(next(a));
        else if (!strcmp(a, "--rc")) lp.rc = atof(next(a));
        else if (!strcmp(a, "--center")) lp.center = atoi(next(a));
        else if (!strcmp(a, "--checkpoint")) ckpt = next(a);
        else if (!strcmp(a, "--dcd")) dcd = true;
        else if (!strcmp(a, "--tune")) tune = true;
        else if (!strcmp(a, "--debye")) debye = atof(next(a));
        else if (a[0] == '-' && a[1] != '-') {
            switch (a[1]) {  // E:6082-6099
            case 'D': lp.ss_D = atof(a + 2); break;
            case 'E': lp.hs_D = atof(a + 2); break;
            case 'd': lp.st_D = atof(a + 2); break;
            case 'T': lp.T = atof(a + 2); break;
            case 'c': lp.c_mg = atof(a + 2); break;
            case 'f': lp.c_k = atof(a + 2); break;
            case 's': lp.seed = atoi(a + 2); break;
            default: printf("unrecognized argument %s\n", a); break;
            }
        } else {
            printf("unrecognized argument %s\n", a);
        }
    }
    if (replicas < 1 || every < 1 || steps < 0) {
        fprintf(stderr, "tis_run: bad --replicas/--every/--steps\n");
        return 2;
    }

    // set-up (E:6111-6179) of every replica, then the restart read (E:6181-6211)
    std::vector<tis_system *> sys(replicas, nullptr);
    std::vector<Names> files(replicas);
    const int seed0 = lp.seed;
    for (int r = 0; r < replicas; ++r) {
        tis_load_params q = lp;
        q.seed = seed0 + r;
        if (report(tis_system_load(&q, &sys[r]), "set-up")) return 1;
        if (debye != 0.0 && report(tis_system_set(sys[r], "debye", TIS_F64, &debye, 1), "--debye")) return 1;
        files[r] = names(lp, q.seed);
    }
    if (tune) {
        tis_run_params best;
        // tuned for the loop's calls: one frame interval per tis_step, at most 1000 steps a trial call
        const int64_t per_call = every < 1000 ? every : 1000;
        if (report(tis_autotune(sys.data(), replicas, &rp, per_call, "tis_tune.txt", &best, nullptr), "tune")) return 1;
        rp = best;
    }
    tis_handle *h = nullptr;
    if (report(tis_create(sys.data(), replicas, &rp, &h), "tis_create")) return 1;
    long long klok_old = -1;  // every replica resumes at the same step (the first file's frames)
    bool resumed = false;
    if (!ckpt.empty()) {  // the bit-exact checkpoint and its step (FILE.klok) when present
        FILE *probe = fopen(ckpt.c_str(), "rb");
        if (probe) {
            fclose(probe);
            if (report(tis_checkpoint_load(h, ckpt.c_str()), "checkpoint")) return 1;
            FILE *kf = fopen((ckpt + ".klok").c_str(), "r");
            if (!kf || fscanf(kf, "%lld", &klok_old) != 1) {
                fprintf(stderr, "tis_run: %s.klok missing or unreadable\n", ckpt.c_str());
                return 1;
            }
            fclose(kf);
            resumed = true;
        }
    }
    for (int r = 0; r < replicas && !resumed; ++r) {
        int n = 0;
        tis_replica_size(h, r, &n);
        FILE *probe = fopen(files[r].coordinates.c_str(), "rb");
        if (!probe) {
            if (klok_old > 0) {
                fprintf(stderr, "tis_run: %s missing while other replicas resume\n", files[r].coordinates.c_str());
                return 1;
            }
            klok_old = 0;
            continue;
        }
        fclose(probe);
        std::vector<double> st[9];
        for (auto &v : st) v.resize(n);
        int64_t frames = 0;
        if (report(tis_read_last_frame(files[r].coordinates.c_str(), n, st[0].data(), st[1].data(), st[2].data(),
                                       &frames),
                   "restart"))
            return 1;
        if (klok_old >= 0 && klok_old != frames * every) {
            fprintf(stderr, "tis_run: replicas' output files hold different numbers of frames\n");
            return 1;
        }
        klok_old = frames * every;  // the reference: frames * 10^6, its frame interval
        if (frames == 0) continue;
        // x_old = x - v h with the set-up velocities (E:6203-6209)
        const void *pv[4] = {nullptr, nullptr, nullptr, nullptr};
        int dt = 0;
        int64_t cnt = 0;
        const char *vn[3] = {"vx", "vy", "vz"};
        for (int c = 0; c < 3; ++c)
            if (report(tis_system_get(sys[r], vn[c], &dt, &pv[c], &cnt), "set-up velocities")) return 1;
        const double *vx = (const double *)pv[0], *vy = (const double *)pv[1], *vz = (const double *)pv[2];
        const double step_h =
            (tis_system_get(sys[r], "h", &dt, &pv[3], &cnt) == TIS_OK && pv[3] && dt == TIS_F64) ? ((const double *)pv[3])[0] : 0.05;
        for (int i = 0; i < n; ++i) {
            st[3][i] = st[0][i] - vx[i] * step_h;
            st[4][i] = st[1][i] - vy[i] * step_h;
            st[5][i] = st[2][i] - vz[i] * step_h;
            st[6][i] = vx[i];
            st[7][i] = vy[i];
            st[8][i] = vz[i];
        }
        if (report(tis_set_state(h, r, st[0].data(), st[1].data(), st[2].data(), st[3].data(), st[4].data(),
                                 st[5].data(), st[6].data(), st[7].data(), st[8].data()),
                   "restart state"))
            return 1;
    }
    if (klok_old < 0) klok_old = 0;
    if (!resumed && report(tis_populate_lists(h), "populate_lists")) return 1;
    double step_h = 0.05;
    {
        int dt = 0;
        const void *pv = nullptr;
        int64_t cnt = 0;
        if (tis_system_get(sys[0], "h", &dt, &pv, &cnt) == TIS_OK && pv && dt == TIS_F64) step_h = ((const double *)pv)[0];
    }

    // the run loop (E:6274-6387): a frame at every multiple of `every`, before that step
    const long long end = steps + 1;
    long long klok = klok_old + 1;
    bool skip_frame = resumed;  // a checkpoint is saved after its frame was written
    while (klok < end) {
        if (klok % every == 0 && !skip_frame) {
            if (report(tis_sync(h), "step")) return 1;
            for (int r = 0; r < replicas; ++r) {
                if (report(tis_write_frame(h, r, files[r].contacts.c_str(), files[r].coordinates.c_str(),
                                           files[r].energies.c_str()),
                           "output"))
                    return 1;
                if (dcd) {
                    std::string trj = files[r].coordinates;
                    trj.replace(0, strlen("Coordinates"), "Trajectory");
                    trj.replace(trj.size() - 4, 4, ".dcd");
                    if (report(tis_write_dcd(h, r, trj.c_str(), (int)std::min<long long>(every, 2147483647LL), step_h),
                               "dcd"))
                        return 1;
                }
                if (snap_every > 0 && (klok % snap_every == 0 || klok == end - 1)) {
                    const Names snap = names(lp, seed0 + r, true, klok / snap_every);
                    copy_file(files[r].contacts, snap.contacts);
                    copy_file(files[r].coordinates, snap.coordinates);
                    copy_file(files[r].energies, snap.energies);
                    if (klok != end - 1) {
                        const Names old = names(lp, seed0 + r, true, klok / snap_every - 3);
                        remove(old.contacts.c_str());
                        remove(old.coordinates.c_str());
                        remove(old.energies.c_str());
                    }
                }
            }
        }
        if (!ckpt.empty() && klok % every == 0 && !skip_frame) {  // checkpoint at every frame, replaced atomically
            const std::string tmp = ckpt + ".tmp";
            if (report(tis_checkpoint_save(h, tmp.c_str()), "checkpoint")) return 1;
            FILE *kf = fopen((tmp + ".klok").c_str(), "w");
            if (!kf) {
                fprintf(stderr, "tis_run: cannot write %s.klok\n", tmp.c_str());
                return 1;
            }
            fprintf(kf, "%lld\n", klok - 1);
            fclose(kf);
            if (rename(tmp.c_str(), ckpt.c_str()) != 0 || rename((tmp + ".klok").c_str(), (ckpt + ".klok").c_str()) != 0) {
                fprintf(stderr, "tis_run: cannot replace %s\n", ckpt.c_str());
                return 1;
            }
        }
        skip_frame = false;
        long long next = (klok / every + 1) * every;
        if (next > end) next = end;
        if (report(tis_step(h, next - klok), "step")) return 1;
        klok = next;
    }
    const int rc = report(tis_sync(h), "step");
    tis_destroy(h);
    for (tis_system *s : sys) tis_system_destroy(s);
    return rc ? 1 : 0;
}
