// tis_system_load: reads the reference's four input files and runs its set-up
// (E: = src/16SCD_Mg_Cl_K_COPY_fast.cpp of naotohori/16S-central-folding):
//   read_maxi_key E:2883, read_PDB E:3137, initialize_HB_atoms E:3671,
//   initialize_unprocessed_bonds E:3733, initialize_unprocessed_stacks E:4232,
//   set_box E:4542, ion numbers E:6167-6171, add_crowder E:5055.
// The result is one replica's system in the array layout the engine consumes
// (0-based particle indices; bonded terms in polymer_constraints order).
//
// Values that must round exactly as the reference's (bead centroids, native
// angles and dihedrals, the principal-axis rotation, random velocities and ion
// positions) are computed with the reference's operation order; build this file
// with -ffp-contract=off.  Random draws come from glibc rand() after the same
// srand() call as the reference, or from the Philox stream.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tis_device.cuh"
#include "tis_host.h"

using tis::fail;

namespace {

const double kPi = 3.14159265358979323846264338328;

// force-field tables of the reference (polymer_constraints E:2370-2470, secondary
// stacks E:4399-4429, canonical H-bond geometry E:3967-3986)
struct BaseBonded { char b; double r0, alpha1, alpha2; };
const BaseBonded kBaseBonded[4] = {
    {'A', 4.8515, 1.9259, 1.7029}, {'C', 4.2738, 1.9655, 1.5803},
    {'G', 4.9659, 1.9150, 1.7690}, {'U', 4.2733, 1.9663, 1.5735}};

struct SecStack { char a, b; double r0, e0, div, slope, t0; };
const SecStack kSecStack[16] = {
    {'A', 'A', 4.1806530, -5.194, 0.7093838769, -0.319, 0.594}, {'A', 'C', 3.8260185, -5.146, 0.7185955600, -0.319, 0.594},
    {'A', 'G', 4.4255305, -5.977, 0.6968019829, 5.301, 0.678},  {'A', 'U', 3.8260185, -5.146, 0.7185955600, -0.319, 0.594},
    {'C', 'A', 4.7010580, -5.163, 0.6847830171, -0.319, 0.594}, {'C', 'C', 4.2500910, -4.873, 0.6991615586, -1.567, 0.568},
    {'C', 'G', 4.9790760, -5.482, 0.6816268897, 0.774, 0.627},  {'C', 'U', 4.2273615, -4.873, 0.6832570771, -1.567, 0.568},
    {'G', 'A', 4.0128560, -5.948, 0.6903176657, 5.301, 0.678},  {'G', 'C', 3.6784360, -5.927, 0.7042060343, 4.370, 0.682},
    {'G', 'G', 4.2427250, -6.416, 0.6971421514, 7.346, 0.728},  {'G', 'U', 3.6616930, -5.836, 0.6984426543, 2.924, 0.672},
    {'U', 'A', 4.7010580, -5.163, 0.6847830171, -0.319, 0.594}, {'U', 'C', 4.2679180, -4.880, 0.6758595771, -1.567, 0.568},
    {'U', 'G', 4.9977560, -5.886, 0.7025528229, 2.924, 0.672},  {'U', 'U', 4.2453650, -4.267, 0.6686014771, -3.563, 0.500}};

struct CanGeom { const char *code; double r, t1, t2, p, p1, p2; };
const CanGeom kCan[10] = {
    {"CAN11", 5.8815, 2.7283, 2.5117, 1.2559, 0.9545, 1.1747}, {"CAN12", 5.8815, 2.5117, 2.7283, 1.2559, 1.1747, 0.9545},
    {"CAN21", 5.6550, 2.4837, 2.8230, 1.3902, 1.2174, 0.7619}, {"CAN22", 5.6550, 2.8230, 2.4837, 1.3902, 0.7619, 1.2174},
    {"CAN31", 5.9234, 2.9051, 2.0544, 2.1469, -0.5366, 1.4288}, {"CAN32", 5.9234, 2.0544, 2.9051, 2.1469, 1.4288, -0.5366},
    {"CAN41", 5.3737, 2.8295, 2.0314, 0.6063, 1.0893, 1.4835}, {"CAN42", 5.3737, 2.0314, 2.8295, 0.6063, 1.4835, 1.0893},
    {"CAN51", 6.4922, 2.0579, 1.3569, 3.1147, -1.4796, 1.5278}, {"CAN52", 6.4922, 1.3569, 2.0579, 3.1147, 1.5278, -1.4796}};

// entries whose tertiary-stack excess is reduced by 2 instead of 1 (E:4458-4491)
const int kStExcessTwo[15] = {2 * (583 - 561) - 2, 2 * (587 - 561) - 2, 2 * (658 - 561) - 2, 2 * (687 - 561) - 2,
                              2 * (700 - 561) - 2, 2 * (701 - 561) - 2, 2 * (721 - 561) - 2, 2 * (727 - 561) - 2,
                              2 * (760 - 561) - 2, 2 * (782 - 561) - 2, 2 * (802 - 561) - 2, 2 * (814 - 561) - 2,
                              2 * (881 - 567) - 2, 2 * (892 - 567) - 2, 2 * (898 - 567) - 2};

int residue_index(int res) { return res < 842 ? res - 561 : res - 567; }  // E:3783-3795

struct Setup {
    const tis_load_params *p;
    double T, h = 0.05, lB;
    double MASS[10], RLJ[10], ELJ[10], QC[10];
    // reference-style 1-based arrays
    std::vector<char> amino{0};
    std::vector<int> part{0}, maxi{0};
    std::vector<double> x{0}, y{0}, z{0}, xo{0}, yo{0}, zo{0}, vx{0}, vy{0}, vz{0};
    std::vector<int> ak0{0}, ak1{0};  // atom_key[e][0], atom_key[e][1]
    int NBP = 0, NTP = 0, NT = 0;
    // rand()
    unsigned long long philox_ctr = 0;
    int rnd()
    {
        if (p->rng == 1) return (int)tis::rand_value((unsigned long long)p->seed, philox_ctr++);
        return rand();
    }
    // hydrogen bonds
    std::vector<std::vector<int>> hb_atom_key;  // [entry][j] -> HB atom id (1-based)
    std::vector<int> valence{0};
    std::vector<std::vector<int>> hb_atom_cands{{}};  // HB_ATOM (1-based candidate ids)
    std::vector<int> hk10{0}, hk11{0}, hk12{0}, hk20{0}, hk21{0}, hk22{0}, hdode{0};
    std::vector<double> hr{0}, ht1{0}, ht2{0}, hp{0}, hp1{0}, hp2{0}, hE{0};
    std::vector<double> hdE{0};  // d hb_E / d hs_D of every candidate
    std::vector<std::vector<int>> atom_hb{{}};  // ATOM_HB
    // stacks
    std::vector<int> st_i{0}, st_j{0}, site0{0}, site1{0}, st_excess;
    std::vector<double> sr{0}, st1{0}, st2{0}, sp{0}, sp1{0}, sp2{0}, sE{0};
    std::vector<double> sdss{0};  // d st_E / d ss_D of every stack (0 for tertiary stacks)
    std::vector<int> scls{0};     // 5' base of a secondary stack: 0 A, 1 C, 2 G, 3 U (-1 tertiary)
    int s3N = 0, stN = 0;

    double dist(int i1, int i2) const
    {
        double a = x[i1] - x[i2], b = y[i1] - y[i2], c = z[i1] - z[i2];
        return sqrt(a * a + b * b + c * c);
    }
    double angle(int i1, int i2, int i3) const
    {
        double v1[3] = {x[i1] - x[i2], y[i1] - y[i2], z[i1] - z[i2]};
        double v2[3] = {x[i3] - x[i2], y[i3] - y[i2], z[i3] - z[i2]};
        double n1 = v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2];
        double n2 = v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2];
        double n12 = sqrt(n1 * n2);
        return acos((v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2]) / n12);
    }
    double dihedral(int i1, int i2, int i3, int i4) const
    {
        double v1[3] = {x[i2] - x[i1], y[i2] - y[i1], z[i2] - z[i1]};
        double v2[3] = {x[i3] - x[i2], y[i3] - y[i2], z[i3] - z[i2]};
        double v3[3] = {x[i4] - x[i3], y[i4] - y[i3], z[i4] - z[i3]};
        double m[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
        double n[3] = {v2[1] * v3[2] - v2[2] * v3[1], v2[2] * v3[0] - v2[0] * v3[2], v2[0] * v3[1] - v2[1] * v3[0]};
        double l = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
        double c = m[0] * n[0] + m[1] * n[1] + m[2] * n[2];
        double s = (v1[0] * n[0] + v1[1] * n[1] + v1[2] * n[2]) * l;
        return atan2(s, c);
    }

    // generate_atom_velocity (E:509-566)
    void velocity(int k)
    {
        int l = maxi[k];
        double *v[3] = {&vx[k], &vy[k], &vz[k]};
        for (int c = 0; c < 3; ++c) {
            double a1;
            do a1 = (double)rnd() / RAND_MAX;
            while (a1 == 0);
            double a2 = (double)rnd() / RAND_MAX;
            double t1 = sqrt(T / MASS[l]) * sqrt(-2.0 * log(a1));
            double t2 = 2.0 * kPi * a2;
            *v[c] = t1 * cos(t2);
        }
        xo[k] = x[k] - vx[k] * h;
        yo[k] = y[k] - vy[k] * h;
        zo[k] = z[k] - vz[k] * h;
    }

    int read_maxikey()
    {
        FILE *f = fopen(p->maxikey, "r");
        if (!f) return fail(TIS_ERR_IO, "cannot open %s", p->maxikey);
        for (int t = 1; t <= 9; ++t) {
            int dummy;
            if (fscanf(f, "%d %le %le %le %le\n", &dummy, MASS + t, RLJ + t, ELJ + t, QC + t) != 5) {
                fclose(f);
                return fail(TIS_ERR_FORMAT, "%s: line %d not 'type mass radius depth charge'", p->maxikey, t);
            }
        }
        fclose(f);
        return TIS_OK;
    }

    // read_PDB (E:3137-3632): two token-driven passes over white-space separated fields
    int read_pdb()
    {
        FILE *f = fopen(p->pdb, "r");
        if (!f) return fail(TIS_ERR_IO, "cannot open %s", p->pdb);
        char str[256], junk[256];
        int entry = 0, k = 0;
        do {  // pass 1: residues and their kind
            entry++;
            if (fscanf(f, "%255s", str) != 1) str[0] = 0;
            if (entry == 3) {
                if (!strcmp(str, "P")) amino.push_back('P');
                else if (!strcmp(str, "O5'")) { amino.push_back(0); k = 1; }
            } else if (entry == 4 && k) {
                if (!strcmp(str, "A") || !strcmp(str, "G") || !strcmp(str, "C") || !strcmp(str, "U")) amino.back() = str[0];
                k = 0;
            } else if (entry == 9) {
                if (!fgets(junk, sizeof junk, f)) junk[0] = 0;
                entry = 0;
            }
        } while (!feof(f));
        NBP = (int)amino.size() - 1;
        for (int e = 1; e <= NBP; ++e)
            if (amino[e] == 0) {
                fclose(f);
                return fail(TIS_ERR_FORMAT, "%s: residue %d is not A, C, G or U", p->pdb, e);
            }
        ak0.assign(NBP + 2, 0);
        ak1.assign(NBP + 2, 0);
        rewind(f);
        int i = 0, j = 0;
        k = 0;
        entry = 0;
        auto new_bead = [&](int kind_, int maxi_) {
            NT += 1;
            part.push_back(kind_);
            maxi.push_back(maxi_);
            x.push_back(0); y.push_back(0); z.push_back(0);
        };
        do {  // pass 2: bead centroids
            entry++;
            if (fscanf(f, "%255s", str) != 1) str[0] = 0;
            if (entry == 3) {
                if (!strcmp(str, "P")) {
                    j = 0;
                    x[NT] /= i; y[NT] /= i; z[NT] /= i;
                    k += 1;
                    new_bead(0, 1);
                    ak0[k] = NT;
                    i = 1;
                } else if (!strcmp(str, "O5'")) {
                    if (i) { x[NT] /= i; y[NT] /= i; z[NT] /= i; }
                    k += 1;
                    new_bead(1, 2);
                    ak0[k] = NT;
                    i = 1;
                } else if ((!strcmp(str, "N9") && (amino[k] == 'A' || amino[k] == 'G')) ||
                           (!strcmp(str, "N1") && (amino[k] == 'C' || amino[k] == 'U'))) {
                    x[NT] /= i; y[NT] /= i; z[NT] /= i;
                    const int mk = amino[k] == 'A' ? 3 : amino[k] == 'G' ? 4 : amino[k] == 'C' ? 5 : 6;
                    new_bead(2, mk);
                    ak1[k] = NT;
                    i = 1;
                } else if (str[0] != 'H') {
                    i++;
                } else {
                    j = 1;
                }
            } else if (entry == 7) {
                if (!j) x[NT] += atof(str);
            } else if (entry == 8) {
                if (!j) y[NT] += atof(str);
            } else if (entry == 9) {
                if (!j) z[NT] += atof(str);
                if (!fgets(junk, sizeof junk, f)) junk[0] = 0;
                entry = 0;
            }
        } while (!feof(f));
        fclose(f);
        x[NT] /= i; y[NT] /= i; z[NT] /= i;
        if (NT < 3 || NBP < 3) return fail(TIS_ERR_FORMAT, "%s: fewer than three backbone entries", p->pdb);
        if (amino[1] == 'P') return fail(TIS_ERR_FORMAT, "%s: the chain must start with a nucleotide (no 5' phosphate)", p->pdb);
        NTP = NT;
        xo.assign(NT + 1, 0); yo.assign(NT + 1, 0); zo.assign(NT + 1, 0);
        vx.assign(NT + 1, 0); vy.assign(NT + 1, 0); vz.assign(NT + 1, 0);
        for (int e = 1; e <= NBP; ++e) {  // E:3621-3625, entry by entry, site 0 then 1
            velocity(ak0[e]);
            if (amino[e] != 'P') velocity(ak1[e]);
        }
        return TIS_OK;
    }

    // initialize_HB_atoms (E:3671-3729)
    void hb_atoms()
    {
        hb_atom_key.assign(NBP + 2, {});
        int id = 0;
        for (int e = 1; e <= NBP; ++e) {
            int ns, a, b, c;
            switch (amino[e]) {
                case 'A': ns = 5; a = 4; b = 0; c = -1; break;
                case 'C': ns = 4; a = 4; b = 0; c = 2; break;
                case 'G': ns = 6; a = 3; b = 0; c = 5; break;
                case 'U': ns = 4; a = -1; b = 0; c = 2; break;
                default: ns = 1; a = -1; b = -1; c = -1; break;  // P
            }
            for (int jj = 0; jj <= ns; ++jj) {
                ++id;
                hb_atom_key[e].push_back(id);
                valence.push_back((jj == a || jj == b || jj == c) ? 2 : 1);
                hb_atom_cands.emplace_back();
            }
        }
    }

    // return_HB_JNDX (E:3636-3667); -1 for a name the reference does not map
    static int hb_jndx(const char *atom, char nuc)
    {
        int j = -1;
        if (!strcmp(atom, "N1")) j = 2;
        if (!strcmp(atom, "N2")) j = 3;
        if (!strcmp(atom, "N3")) j = (nuc == 'G') ? 4 : 3;
        if (!strcmp(atom, "N4")) j = 4;
        if (!strcmp(atom, "N6")) j = 4;
        if (!strcmp(atom, "N7")) { if (nuc == 'A') j = 5; if (nuc == 'G') j = 6; }
        if (!strcmp(atom, "O2")) j = 2;
        if (!strcmp(atom, "O4")) j = 4;
        if (!strcmp(atom, "O6")) j = 5;
        if (!strcmp(atom, "O2'")) j = 0;
        if (!strcmp(atom, "O4'")) j = 1;
        if (!strcmp(atom, "OP1")) j = 0;
        if (!strcmp(atom, "OP2")) j = 1;
        return j;
    }

    bool entry_ok(int e) const { return e >= 1 && e <= NBP; }

    // the three beads an H-bonding atom name selects (E:3805-3852)
    bool triple(const char *A, int RES, int &k0, int &k1, int &k2) const
    {
        int e0, e1, e2;
        bool base = false;
        if (!strcmp(A, "OP1") || !strcmp(A, "OP2")) { e0 = 2 * RES - 1; e1 = 2 * RES - 2; e2 = 2 * RES; }
        else if (!strcmp(A, "O2'") || !strcmp(A, "O4'")) { e0 = 2 * RES; e1 = 2 * RES - 1; e2 = 2 * RES + 1; }
        else { e0 = 2 * RES - 1; e1 = 2 * RES - 1; e2 = 2 * RES; base = true; }
        if (!entry_ok(e0) || !entry_ok(e1) || !entry_ok(e2)) return false;
        k0 = ak0[e0];
        k1 = base ? ak1[e1] : ak0[e1];
        k2 = ak0[e2];
        return k0 > 0 && k1 > 0 && k2 > 0;
    }

    // initialize_unprocessed_bonds (E:3733-4119)
    int read_bonds()
    {
        FILE *f = fopen(p->bonds, "r");
        if (!f) return fail(TIS_ERR_IO, "cannot open %s", p->bonds);
        char A0[64], A01[64], A02[64], A1[64], A2[64];
        int bpN = 0;
        do {  // record count (E:3752-3760)
            bpN += 1;
            int guard = 0;
            do {
                if (fscanf(f, "%63s", A1) != 1) {
                    fclose(f);
                    return fail(TIS_ERR_FORMAT, "%s: record %d does not end with TER before the end of the file "
                                "(the reference's reader also needs no newline after the last TER)", p->bonds, bpN);
                }
            } while (strcmp(A1, "TER") != 0 && ++guard < 1000);
        } while (!feof(f));
        rewind(f);
        int hbN = 0;
        for (int rec = 1; rec <= bpN; ++rec) {
            const int kmin = hbN;
            if (fscanf(f, "%63s %63s %63s %63s", A0, A01, A02, A1) != 4) {
                fclose(f);
                return fail(TIS_ERR_FORMAT, "%s: record %d truncated", p->bonds, rec);
            }
            const int RES1 = residue_index(atoi(A01)), RES2 = residue_index(atoi(A02));
            do {
                if (fscanf(f, "%63s", A2) != 1) {
                    fclose(f);
                    return fail(TIS_ERR_FORMAT, "%s: record %d truncated", p->bonds, rec);
                }
                int k10, k11, k12, k20, k21, k22;
                if (!triple(A1, RES1, k10, k11, k12) || !triple(A2, RES2, k20, k21, k22)) {
                    fclose(f);
                    return fail(TIS_ERR_FORMAT, "%s: record %d names a bead outside the chain", p->bonds, rec);
                }
                int k = kmin + 1;
                for (; k <= hbN; ++k)
                    if (k10 == hk10[k] && k11 == hk11[k] && k12 == hk12[k] && k20 == hk20[k] && k21 == hk21[k] && k22 == hk22[k])
                        break;
                if (k <= hbN) {
                    hE[k] -= p->hs_D * 0.73753;
                    hdE[k] -= 0.73753;
                } else if ((!strcmp(A0, "CAN51") && !strcmp(A2, "O2'")) || (!strcmp(A0, "CAN52") && !strcmp(A1, "O2'"))) {
                    k = hbN;
                    if (k < 1) {
                        fclose(f);
                        return fail(TIS_ERR_FORMAT, "%s: CAN51/CAN52 O2' pair before any candidate", p->bonds);
                    }
                } else {
                    ++hbN;
                    hk10.push_back(k10); hk11.push_back(k11); hk12.push_back(k12);
                    hk20.push_back(k20); hk21.push_back(k21); hk22.push_back(k22);
                    hr.push_back(dist(k11, k21));
                    ht1.push_back(angle(k10, k11, k21));
                    ht2.push_back(angle(k20, k21, k11));
                    hp.push_back(dihedral(k10, k11, k21, k20));
                    hp1.push_back(dihedral(k21, k11, k10, k12));
                    hp2.push_back(dihedral(k11, k21, k20, k22));
                    hE.push_back(-p->hs_D * 0.73753);
                    hdE.push_back(-0.73753);
                    for (const CanGeom &g : kCan)
                        if (!strcmp(A0, g.code)) {
                            hr[hbN] = g.r; ht1[hbN] = g.t1; ht2[hbN] = g.t2;
                            hp[hbN] = g.p; hp1[hbN] = g.p1; hp2[hbN] = g.p2;
                        }
                    hdode.push_back((!strcmp(A0, "NON00") || !strcmp(A0, "APLAT")) ? 1 : 0);
                    atom_hb.emplace_back();
                    k = hbN;
                }
                const int e1 = (!strcmp(A1, "OP1") || !strcmp(A1, "OP2")) ? 2 * RES1 - 2 : 2 * RES1 - 1;
                const int e2 = (!strcmp(A2, "OP1") || !strcmp(A2, "OP2")) ? 2 * RES2 - 2 : 2 * RES2 - 1;
                const int j1 = hb_jndx(A1, amino[e1]), j2 = hb_jndx(A2, amino[e2]);
                if (j1 < 0 || j2 < 0 || j1 >= (int)hb_atom_key[e1].size() || j2 >= (int)hb_atom_key[e2].size()) {
                    fclose(f);
                    return fail(TIS_ERR_FORMAT, "%s: record %d: atom %s/%s is not an H-bonding atom of its residue", p->bonds, rec, A1, A2);
                }
                const int a1 = hb_atom_key[e1][j1], a2 = hb_atom_key[e2][j2];
                atom_hb[k].push_back(a1);
                atom_hb[k].push_back(a2);
                hb_atom_cands[a1].push_back(k);
                hb_atom_cands[a2].push_back(k);
                if (fscanf(f, "%63s", A1) != 1) {
                    fclose(f);
                    return fail(TIS_ERR_FORMAT, "%s: record %d truncated", p->bonds, rec);
                }
            } while (strcmp(A1, "TER") != 0);
        }
        fclose(f);
        return TIS_OK;
    }

    // initialize_unprocessed_stacks (E:4232-4492)
    int read_stacks()
    {
        FILE *f = fopen(p->stacks, "r");
        if (!f) return fail(TIS_ERR_IO, "cannot open %s", p->stacks);
        st_excess.assign(NBP + 2, 0);
        fseek(f, 0L, SEEK_END);
        const long finish = ftell(f);
        fseek(f, 0L, SEEK_SET);
        if (finish <= 0) {
            fclose(f);
            return fail(TIS_ERR_FORMAT, "%s: empty (the reference needs at least one tertiary stack)", p->stacks);
        }
        char A1[64], A2[64];
        long pos;
        do {
            if (fscanf(f, "%63s %63s\n", A1, A2) != 2) {
                fclose(f);
                return fail(TIS_ERR_FORMAT, "%s: malformed line", p->stacks);
            }
            const int RES1 = residue_index(atoi(A1 + 1)), RES2 = residue_index(atoi(A2 + 1));
            int i = 2 * RES1 - 1, j = 2 * RES2 - 1;
            if (!entry_ok(i) || !entry_ok(i + 1) || !entry_ok(j) || !entry_ok(j + 1) || amino[i] == 'P' || amino[j] == 'P') {
                fclose(f);
                return fail(TIS_ERR_FORMAT, "%s: stack %s %s outside the chain", p->stacks, A1, A2);
            }
            ++stN;
            const int k10 = ak0[i], k11 = ak1[i], k12 = ak0[i + 1], k20 = ak0[j], k21 = ak1[j], k22 = ak0[j + 1];
            st_i.push_back(i);
            st_j.push_back(j);
            sr.push_back(dist(k11, k21));
            st1.push_back(angle(k10, k11, k21));
            st2.push_back(angle(k20, k21, k11));
            sp.push_back(dihedral(k10, k11, k21, k20));
            sp1.push_back(dihedral(k21, k11, k10, k12));
            sp2.push_back(dihedral(k11, k21, k20, k22));
            sE.push_back(-p->st_D);
            sdss.push_back(0.0);
            scls.push_back(-1);
            if (A1[0] == '-') i--;
            if (A2[0] == '-') j--;
            if (i < 1 || j < 1) {
                fclose(f);
                return fail(TIS_ERR_FORMAT, "%s: '-' site before the first phosphate", p->stacks);
            }
            site0.push_back(i);
            site1.push_back(j);
            st_excess[i] += 1;
            st_excess[j] += 1;
            pos = ftell(f);
        } while (pos < finish);
        fclose(f);
        s3N = stN;
        for (int i = 3; i < NBP - 2; i += 2) {  // secondary stacks (E:4385-4448)
            ++stN;
            st_i.push_back(i);
            st_j.push_back(0);
            double r0 = 0, e = 0, de = 0;
            for (const SecStack &t : kSecStack)
                if (amino[i] == t.a && amino[i + 2] == t.b) {
                    r0 = t.r0;
                    e = t.e0 + p->ss_D / t.div + t.slope * (T - t.t0);
                    de = 1.0 / t.div;
                }
            sr.push_back(r0);
            sE.push_back(e);
            sdss.push_back(de);
            scls.push_back(amino[i] == 'A' ? 0 : amino[i] == 'C' ? 1 : amino[i] == 'G' ? 2 : amino[i] == 'U' ? 3 : -1);
            st1.push_back(0); st2.push_back(0); sp.push_back(0); sp1.push_back(0); sp2.push_back(0);
            site0.push_back(i);
            site1.push_back(i + 1);
            st_excess[i] += 1;
            st_excess[i + 1] += 1;
        }
        for (int e = 1; e <= NBP; ++e) {
            bool two = false;
            for (int t : kStExcessTwo) two |= (e == t);
            st_excess[e] -= two ? 2 : 1;
        }
        return TIS_OK;
    }

    // set_box (E:4542-5051): principal axes of the RNA, then the centre bead to the box centre
    int set_box(int kh, double side)
    {
        double a0 = 0, a1 = 0, a2 = 0;
        for (int i = 1; i <= NTP; ++i) { a0 += x[i]; a1 += y[i]; a2 += z[i]; }
        a0 /= NTP; a1 /= NTP; a2 /= NTP;
        double A = 0, B = 0, C = 0, F = 0, G = 0, H = 0;
        for (int i = 1; i <= NTP; ++i) {
            const double dx = x[i] - a0, dy = y[i] - a1, dz = z[i] - a2;
            A += dy * dy + dz * dz;
            B += dx * dx + dz * dz;
            C += dx * dx + dy * dy;
            F += dy * dz;
            G += dx * dz;
            H += dx * dy;
        }
        double n1[3], n2[3], n3[3];
        double *ep1 = nullptr, *ep2 = nullptr, *ep3 = nullptr;
        double x_min, y_min, z_min, x_max, y_max, z_max;
        // order two in-plane eigenpairs and the axis eigenpair (shared tail of the special cases)
        auto order = [&](double e1, double e2, double e3) {
            if (e1 < e2) { x_min = e1; y_min = e2; ep1 = n1; ep2 = n2; }
            else { x_min = e2; y_min = e1; ep1 = n2; ep2 = n1; }
            if (e3 < x_min) { z_min = y_min; y_min = x_min; x_min = e3; ep3 = ep2; ep2 = ep1; ep1 = n3; }
            else if (e3 < y_min) { z_min = y_min; y_min = e3; ep3 = ep2; ep2 = n3; }
            else { z_min = e3; ep3 = n3; }
            if (ep1[0] < 0) { ep1[0] = -ep1[0]; ep1[1] = -ep1[1]; ep1[2] = -ep1[2]; }
            if (ep2[1] < 0) { ep2[0] = -ep2[0]; ep2[1] = -ep2[1]; ep2[2] = -ep2[2]; }
        };
        auto unit = [](double *v) {
            const double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            v[0] /= l; v[1] /= l; v[2] /= l;
        };
        if (fabs(F) < 1.0e-6 && fabs(G) < 1.0e-6) {
            a0 = sqrt(B * B - 2.0 * A * B + A * A + 4.0 * H * H);
            x_max = 0.5 * (B + A + a0);
            n1[0] = 0.5 * (B - A - a0) / H; n1[1] = 1; n1[2] = 0; unit(n1);
            y_max = 0.5 * (B + A - a0);
            n2[0] = 0.5 * (B - A + a0) / H; n2[1] = 1; n2[2] = 0; unit(n2);
            z_max = C;
            n3[0] = 0; n3[1] = 0; n3[2] = 1;
            order(x_max, y_max, z_max);
        } else if (fabs(F) < 1.0e-6 && fabs(H) < 1.0e-6) {
            a0 = sqrt(C * C - 2.0 * A * C + A * A + 4.0 * G * G);
            x_max = 0.5 * (C + A + a0);
            n1[0] = 0.5 * (C - A - a0) / G; n1[1] = 0; n1[2] = 1; unit(n1);
            y_max = 0.5 * (C + A - a0);
            n2[0] = 0.5 * (C - A + a0) / G; n2[1] = 0; n2[2] = 1; unit(n2);
            z_max = B;
            n3[0] = 0; n3[1] = 1; n3[2] = 0;
            order(x_max, y_max, z_max);
        } else if (fabs(G) < 1.0e-6 && fabs(H) < 1.0e-6) {
            a0 = sqrt(C * C - 2.0 * B * C + B * B + 4.0 * F * F);
            x_max = 0.5 * (C + B + a0);
            n1[0] = 0; n1[1] = 0.5 * (C - B - a0) / F; n1[2] = 1; unit(n1);
            y_max = 0.5 * (C + B - a0);
            n2[0] = 0; n2[1] = 0.5 * (C - B + a0) / F; n2[2] = 1; unit(n2);
            z_max = A;
            n3[0] = 1; n3[1] = 0; n3[2] = 0;
            order(x_max, y_max, z_max);
        } else {
            // general case: eigenvalues of the inertia tensor by the trigonometric
            // solution of its characteristic cubic, eigenvectors by ratios
            a2 = -A - B - C;
            a1 = A * B + A * C + B * C - H * H - G * G - F * F;
            a0 = A * F * F + B * G * G + C * H * H + 2.0 * H * G * F - A * B * C;
            x_min = -a2 / 3.0;
            x_max = (9.0 * a1 * a2 - 27 * a0 - 2.0 * a2 * a2 * a2) / 54.0;
            y_max = x_min * x_min - a1 / 3.0;
            y_min = 2.0 * sqrt(y_max);
            z_min = acos(x_max * pow(y_max, -1.5)) / 3.0;
            a0 = kPi / 3.0;
            x_max = x_min + y_min * cos(z_min);
            y_max = x_min - y_min * cos(z_min - a0);
            z_max = x_min - y_min * cos(z_min + a0);
            if (x_max < y_max) { x_min = x_max; y_min = y_max; }
            else { x_min = y_max; y_min = x_max; }
            if (z_max < x_min) { z_min = y_min; y_min = x_min; x_min = z_max; }
            else if (z_max < y_min) { z_min = y_min; y_min = z_max; }
            else z_min = z_max;
            x_max = (A - x_min) * F + G * H;
            y_max = (B - x_min) * G + F * H;
            z_max = (C - x_min) * H + G * F;
            a0 = x_max / y_max;
            a1 = x_max / z_max;
            a2 = sqrt(1.0 + a0 * a0 + a1 * a1);
            n1[0] = 1.0 / a2; n1[1] = a0 / a2; n1[2] = a1 / a2;
            ep1 = n1;
            x_max = (A - y_min) * F + G * H;
            y_max = (B - y_min) * G + F * H;
            z_max = (C - y_min) * H + G * F;
            a0 = y_max / x_max;
            a1 = y_max / z_max;
            a2 = sqrt(1.0 + a0 * a0 + a1 * a1);
            n2[0] = a0 / a2; n2[1] = 1.0 / a2; n2[2] = a1 / a2;
            ep2 = n2;
            ep3 = n3;
        }
        ep3[0] = ep1[1] * ep2[2] - ep1[2] * ep2[1];
        ep3[1] = ep1[2] * ep2[0] - ep1[0] * ep2[2];
        ep3[2] = ep1[0] * ep2[1] - ep1[1] * ep2[0];
        for (int i = 1; i <= NTP; ++i) {
            const double u = x[i] * ep1[0] + y[i] * ep1[1] + z[i] * ep1[2];
            const double v = x[i] * ep2[0] + y[i] * ep2[1] + z[i] * ep2[2];
            const double w = x[i] * ep3[0] + y[i] * ep3[1] + z[i] * ep3[2];
            x[i] = u; y[i] = v; z[i] = w;
        }
        const double half = 0.5 * side;
        const double sx = half - x[kh], sy = half - y[kh], sz = half - z[kh];
        for (int i = 1; i <= NTP; ++i) {
            x[i] += sx; y[i] += sy; z[i] += sz;
            const double u = xo[i] * ep1[0] + yo[i] * ep1[1] + zo[i] * ep1[2] + sx;
            const double v = xo[i] * ep2[0] + yo[i] * ep2[1] + zo[i] * ep2[2] + sy;
            const double w = xo[i] * ep3[0] + yo[i] * ep3[1] + zo[i] * ep3[2] + sz;
            xo[i] = u; yo[i] = v; zo[i] = w;
            const double a = vx[i] * ep1[0] + vy[i] * ep1[1] + vz[i] * ep1[2];
            const double b = vx[i] * ep2[0] + vy[i] * ep2[1] + vz[i] * ep2[2];
            const double c = vx[i] * ep3[0] + vy[i] * ep3[1] + vz[i] * ep3[2];
            vx[i] = a; vy[i] = b; vz[i] = c;
        }
        return TIS_OK;
    }

    // add_crowder (E:5055-5477) for single-site ions: uniform position, rejection on overlap
    int add_ions(int tp, int count, double side)
    {
        const int kind_ = tp == 0 ? 3 : tp == 1 ? 4 : 5;
        const int mk = tp == 0 ? 7 : tp == 1 ? 8 : 9;
        const double hs = 0.5 * side;
        // overlap distances (E:2930)
        double ov[10][10];
        for (int a = 1; a <= 9; ++a)
            for (int b = 1; b <= 9; ++b) {
                const double Dl = (a <= 6 && b <= 6) ? 3.2 : RLJ[a] + RLJ[b];
                ov[a][b] = (Dl - 0.2 * 1.5852) * (Dl - 0.2 * 1.5852);
            }
        for (int c = 0; c < count; ++c) {
            NT += 1;
            part.push_back(kind_);
            maxi.push_back(mk);
            x.push_back(0); y.push_back(0); z.push_back(0);
            xo.push_back(0); yo.push_back(0); zo.push_back(0);
            vx.push_back(0); vy.push_back(0); vz.push_back(0);
            long round = 0;
            for (;;) {
                if (++round > 10000000L) return fail(TIS_ERR_SETUP, "ion placement did not converge (ion %d of type %d)", c + 1, tp);
                double t1 = (double)rnd() / RAND_MAX * side;
                double t2 = (double)rnd() / RAND_MAX * side;
                double t3 = (double)rnd() / RAND_MAX * side;
                double n1[3], n2[3], n3[3];
                for (int d = 0; d < 3; ++d) {  // random unit vector (E:5381-5413)
                    n1[d] = rnd();
                    if ((double)rnd() / RAND_MAX > 0.5) n1[d] = -n1[d];
                }
                double l = sqrt(n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2]);
                n1[0] /= l; n1[1] /= l; n1[2] /= l;
                for (int d = 0; d < 3; ++d) {  // generate_perpendicular_vector (E:433-453)
                    n2[d] = (double)rnd() / RAND_MAX;
                    if ((double)rnd() / RAND_MAX > 0.5) n2[d] = -n2[d];
                }
                double pp = n2[0] * n1[0] + n2[1] * n1[1] + n2[2] * n1[2];
                n2[0] = n2[0] - pp * n1[0]; n2[1] = n2[1] - pp * n1[1]; n2[2] = n2[2] - pp * n1[2];
                pp = sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
                n2[0] = n2[0] / pp; n2[1] = n2[1] / pp; n2[2] = n2[2] / pp;
                n3[0] = n1[1] * n2[2] - n1[2] * n2[1];
                n3[1] = n1[2] * n2[0] - n1[0] * n2[2];
                n3[2] = n1[0] * n2[1] - n1[1] * n2[0];
                // a single-site ion sits at its body origin (RX = RY = RZ = 0, E:2990-3000)
                x[NT] = t1 + n1[0] * 0.0 + n2[0] * 0.0 + n3[0] * 0.0;
                y[NT] = t2 + n1[1] * 0.0 + n2[1] * 0.0 + n3[1] * 0.0;
                z[NT] = t3 + n1[2] * 0.0 + n2[2] * 0.0 + n3[2] * 0.0;
                bool overlap = false;
                for (int k2 = 1; k2 < NT && !overlap; ++k2) {
                    double a = x[NT] - x[k2], b = y[NT] - y[k2], e = z[NT] - z[k2];
                    if (a > hs) a = a - side;
                    if (a < -hs) a = a + side;
                    if (b > hs) b = b - side;
                    if (b < -hs) b = b + side;
                    if (e > hs) e = e - side;
                    if (e < -hs) e = e + side;
                    if (a * a + b * b + e * e < ov[mk][maxi[k2]]) overlap = true;
                }
                if (!overlap) break;
            }
            velocity(NT);
        }
        return TIS_OK;
    }
};

}  // namespace

extern "C" {

int tis_load_params_default(tis_load_params *p)
{
    if (!p) return fail(TIS_ERR_ARG, "null params");
    memset(p, 0, sizeof *p);
    p->T = 0.615;
    p->ss_D = 0.850;
    p->hs_D = 3.975;
    p->st_D = 6.5;
    p->seed = 1;
    p->box = 350.0;
    p->rc = 50.0;
    p->c_mg = 0.005;
    p->c_k = 0.050;
    p->n_mg = p->n_cl = p->n_k = -1;
    p->center = 500;
    p->rng = 0;
    return TIS_OK;
}

int tis_system_load(const tis_load_params *p, tis_system **out)
{
    tis::clear_error();
    if (!p || !out || !p->pdb || !p->bonds || !p->stacks || !p->maxikey) return fail(TIS_ERR_ARG, "tis_system_load: bad argument");
    if (!(p->box > 0) || !(p->T > 0)) return fail(TIS_ERR_ARG, "tis_system_load: box and T must be positive");
    Setup S;
    S.p = p;
    S.T = p->T;
    if (p->rng == 0) srand((unsigned)(p->T * 1000 * p->seed));  // E:6105
    S.lB = 332.0637090 * (0.03273600947 * S.T - 0.00669625750);  // E:6109
    int rc;
    if ((rc = S.read_maxikey())) return rc;
    if ((rc = S.read_pdb())) return rc;
    S.hb_atoms();
    if ((rc = S.read_bonds())) return rc;
    if ((rc = S.read_stacks())) return rc;
    if (p->center < 1 || p->center > S.NTP) return fail(TIS_ERR_ARG, "centre bead %d outside the RNA (1..%d)", p->center, S.NTP);
    S.set_box(p->center, p->box);
    int nion[3];
    if (p->n_mg >= 0 || p->n_cl >= 0 || p->n_k >= 0) {
        nion[0] = p->n_mg < 0 ? 0 : p->n_mg;
        nion[1] = p->n_cl < 0 ? 0 : p->n_cl;
        nion[2] = p->n_k < 0 ? 0 : p->n_k;
    } else {  // E:6167-6171
        const double vol = p->box * p->box * p->box;
        nion[0] = (int)(p->c_mg * 6.022 * 0.0001 * vol);
        nion[2] = (int)(p->c_k * 6.022 * 0.0001 * vol);
        nion[1] = 2 * nion[0] + nion[2] - (S.NBP - 1) / 2;
        if (nion[1] < 0) nion[1] = 0;
    }
    for (int t = 0; t < 3; ++t)
        if ((rc = S.add_ions(t, nion[t], p->box))) return rc;

    tis_system *s = new tis_system();
    const int N = S.NT;
    s->set_i64("n_particles", N);
    s->set_i64("n_rna", S.NTP);
    s->set_i64("n_entries", S.NBP);
    s->set_i64("center", p->center - 1);
    s->set_i64("seed", p->seed);
    s->set_f64("box", {p->box, p->box, p->box});
    s->set_scalar("T", S.T);
    s->set_scalar("h", S.h);
    s->set_scalar("lB", S.lB);
    s->set_scalar("rc", p->rc);
    s->set_scalar("ss_D", p->ss_D);
    s->set_scalar("hs_D", p->hs_D);
    s->set_scalar("st_D", p->st_D);
    s->set_i32("n_ions", {nion[0], nion[1], nion[2]});
    std::vector<int32_t> type(N), kind(N);
    for (int i = 0; i < N; ++i) { type[i] = S.maxi[i + 1]; kind[i] = S.part[i + 1]; }
    s->set_i32("type", type);
    s->set_i32("kind", kind);
    s->set_f64("mass", std::vector<double>(S.MASS + 1, S.MASS + 10));
    s->set_f64("rlj", std::vector<double>(S.RLJ + 1, S.RLJ + 10));
    s->set_f64("elj", std::vector<double>(S.ELJ + 1, S.ELJ + 10));
    s->set_f64("qc", std::vector<double>(S.QC + 1, S.QC + 10));
    std::vector<int32_t> ec(S.NBP), e0(S.NBP), e1(S.NBP);
    for (int e = 1; e <= S.NBP; ++e) {
        ec[e - 1] = S.amino[e];
        e0[e - 1] = S.ak0[e] - 1;
        e1[e - 1] = S.amino[e] == 'P' ? -1 : S.ak1[e] - 1;
    }
    s->set_i32("entry_code", ec);
    s->set_i32("entry_a0", e0);
    s->set_i32("entry_a1", e1);

    // bonded terms in polymer_constraints order (E:2360-2520)
    std::vector<int32_t> bk, ba, bb, bc;
    std::vector<double> bk0, bx0;
    auto bond = [&](int i, int j, double k0, double r0) {
        bk.push_back(0); ba.push_back(i - 1); bb.push_back(j - 1); bc.push_back(-1); bk0.push_back(k0); bx0.push_back(r0);
    };
    auto angle = [&](int i, int j, int k, double k0, double t0) {
        bk.push_back(1); ba.push_back(i - 1); bb.push_back(j - 1); bc.push_back(k - 1); bk0.push_back(k0); bx0.push_back(t0);
    };
    const int NBP = S.NBP;
    for (int e = 1; e <= NBP; e += 2) {
        const BaseBonded *bp = nullptr;
        for (const BaseBonded &t : kBaseBonded)
            if (t.b == S.amino[e]) bp = &t;
        if (!bp) continue;
        const int i = S.ak0[e], j = S.ak1[e];
        bond(i, j, 10.0, bp->r0);
        if (e < NBP) angle(j, i, S.ak0[e + 1], 5.0, bp->alpha1);
        if (e > 1) angle(j, i, S.ak0[e - 1], 5.0, bp->alpha2);
    }
    for (int e = 2; e <= NBP; e += 2) {
        bond(S.ak0[e], S.ak0[e - 1], 64.0, 3.8157);
        if (e > 2) angle(S.ak0[e], S.ak0[e - 1], S.ak0[e - 2], 20.0, 1.4440);
    }
    for (int e = 3; e <= NBP; e += 2) {
        bond(S.ak0[e], S.ak0[e - 1], 23.0, 4.6010);
        angle(S.ak0[e], S.ak0[e - 1], S.ak0[e - 2], 20.0, 1.5256);
    }
    s->set_i32("bt_kind", bk);
    s->set_i32("bt_a", ba);
    s->set_i32("bt_b", bb);
    s->set_i32("bt_c", bc);
    s->set_f64("bt_k0", bk0);
    s->set_f64("bt_x0", bx0);

    // stacks
    {
        const int n3 = S.s3N, n2 = S.stN - S.s3N;
        std::vector<int32_t> idx3, site, si3, sj3, idx2, si2, ex, cls2;
        std::vector<double> nat3, E3, r02, E2, dss2;
        for (int k = 1; k <= n3; ++k) {
            const int i = S.st_i[k], j = S.st_j[k];
            si3.push_back(i); sj3.push_back(j);
            const int ids[6] = {S.ak0[i], S.ak1[i], S.ak0[i + 1], S.ak0[j], S.ak1[j], S.ak0[j + 1]};
            for (int c = 0; c < 6; ++c) idx3.push_back(ids[c] - 1);
            const double nat[6] = {S.sr[k], S.st1[k], S.st2[k], S.sp[k], S.sp1[k], S.sp2[k]};
            for (int c = 0; c < 6; ++c) nat3.push_back(nat[c]);
            E3.push_back(S.sE[k]);
            site.push_back(S.site0[k]);
            site.push_back(S.site1[k]);
        }
        for (int k = S.s3N + 1; k <= S.stN; ++k) {
            const int i = S.st_i[k];
            si2.push_back(i);
            const int ids[7] = {S.ak0[i - 1], S.ak0[i], S.ak1[i], S.ak0[i + 1], S.ak0[i + 2], S.ak1[i + 2], S.ak0[i + 3]};
            for (int c = 0; c < 7; ++c) idx2.push_back(ids[c] - 1);
            r02.push_back(S.sr[k]);
            E2.push_back(S.sE[k]);
            dss2.push_back(S.sdss[k]);
            cls2.push_back(S.scls[k]);
        }
        for (int e = 1; e <= NBP; ++e) ex.push_back(S.st_excess[e]);
        std::vector<int32_t> off(2 * n3, -1);
        for (int t = 0; t < 2 * n3; ++t) {  // E:1960-1981
            const int e = site[t];
            if (S.st_excess[e] == 1) {
                const int idx = (int)ceil(0.5 * e) - 2;
                if (idx >= 0 && idx < n2) off[t] = idx;
            }
        }
        s->set_i32("st3_entry_i", si3);
        s->set_i32("st3_entry_j", sj3);
        s->set_i32("st3_idx", idx3);
        s->set_f64("st3_native", nat3);
        s->set_f64("st3_E", E3);
        s->set_i32("st3_site", site);
        s->set_i32("st_excess", ex);
        s->set_i32("st3_off", off);
        s->set_i32("st2_entry_i", si2);
        s->set_i32("st2_idx", idx2);
        s->set_f64("st2_r0", r02);
        s->set_f64("st2_E", E2);
        s->set_f64("st2_dss", dss2);
        s->set_i32("st2_cls", cls2);
    }
    // hydrogen bonds
    {
        const int nh = (int)S.hE.size() - 1;
        std::vector<int32_t> idx, dode, aoff{0}, aidx, val, coff{0}, cidx;
        std::vector<double> nat, E, dE;
        for (int k = 1; k <= nh; ++k) {
            const int ids[6] = {S.hk10[k], S.hk11[k], S.hk12[k], S.hk20[k], S.hk21[k], S.hk22[k]};
            for (int c = 0; c < 6; ++c) idx.push_back(ids[c] - 1);
            const double nv[6] = {S.hr[k], S.ht1[k], S.ht2[k], S.hp[k], S.hp1[k], S.hp2[k]};
            for (int c = 0; c < 6; ++c) nat.push_back(nv[c]);
            E.push_back(S.hE[k]);
            dE.push_back(S.hdE[k]);
            dode.push_back(S.hdode[k]);
            for (int a : S.atom_hb[k]) aidx.push_back(a - 1);
            aoff.push_back((int32_t)aidx.size());
        }
        const int na = (int)S.valence.size() - 1;
        for (int a = 1; a <= na; ++a) {
            val.push_back(S.valence[a]);
            for (int k : S.hb_atom_cands[a]) cidx.push_back(k - 1);
            coff.push_back((int32_t)cidx.size());
        }
        s->set_i32("hb_idx", idx);
        s->set_f64("hb_native", nat);
        s->set_f64("hb_E", E);
        s->set_f64("hb_dhs", dE);
        s->set_i32("hb_dode", dode);
        s->set_i32("hb_atom_off", aoff);
        s->set_i32("hb_atom_idx", aidx);
        s->set_i32("hba_valence", val);
        s->set_i32("hba_cand_off", coff);
        s->set_i32("hba_cand_idx", cidx);
    }
    std::vector<double> buf(N);
    const std::vector<double> *src[9] = {&S.x, &S.y, &S.z, &S.xo, &S.yo, &S.zo, &S.vx, &S.vy, &S.vz};
    const char *names[9] = {"x", "y", "z", "ox", "oy", "oz", "vx", "vy", "vz"};
    for (int c = 0; c < 9; ++c) {
        for (int i = 0; i < N; ++i) buf[i] = (*src[c])[i + 1];
        s->set_f64(names[c], buf);
    }
    *out = s;
    return TIS_OK;
}

}  // extern "C"
