// The reference's output files (E:6276-6312) and its restart read (E:6181-6211).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>

#include "tis_host.h"

using tis::fail;

extern "C" {

int tis_write_frame(tis_handle *h, int replica, const char *contacts, const char *coordinates, const char *energies)
{
    if (!h) return fail(TIS_ERR_ARG, "null handle");
    int n = 0, rc;
    if ((rc = tis_replica_size(h, replica, &n))) return rc;
    int64_t n3 = 0;
    if ((rc = tis_get_stack_energies(h, replica, nullptr, 0, &n3))) return rc;
    std::vector<double> st(n3 > 0 ? n3 : 1), x(n), y(n), z(n);
    double e5[5];
    if ((rc = tis_get_stack_energies(h, replica, st.data(), n3, &n3))) return rc;
    if ((rc = tis_get_energies(h, replica, e5))) return rc;
    if ((rc = tis_get_state(h, replica, x.data(), y.data(), z.data(), nullptr, nullptr, nullptr, nullptr, nullptr,
                            nullptr)))
        return rc;
    if (contacts) {  // E:6290-6294: every tertiary stack's energy, "%+.3f " each
        FILE *f = fopen(contacts, "a");
        if (!f) return fail(TIS_ERR_IO, "cannot open %s", contacts);
        for (int64_t k = 0; k < n3; ++k) fprintf(f, "%+.3f ", st[k]);
        fprintf(f, "\n");
        fclose(f);
    }
    if (coordinates) {  // E:6298-6304: x, y, z as the 1-based arrays (index 0 unused, written as 0)
        FILE *f = fopen(coordinates, "ab");
        if (!f) return fail(TIS_ERR_IO, "cannot open %s", coordinates);
        const double zero = 0.0;
        bool ok = true;
        for (const std::vector<double> *a : {&x, &y, &z}) {
            ok = ok && fwrite(&zero, sizeof(double), 1, f) == 1;
            ok = ok && fwrite(a->data(), sizeof(double), (size_t)n, f) == (size_t)n;
        }
        fclose(f);
        if (!ok) return fail(TIS_ERR_IO, "short write to %s", coordinates);
    }
    if (energies) {  // E:6308-6312: E2_HB E3_HB E2_STACK E3_STACK Rg, E3_STACK summed from the stacks
        FILE *f = fopen(energies, "a");
        if (!f) return fail(TIS_ERR_IO, "cannot open %s", energies);
        double e3 = 0;
        for (int64_t k = 0; k < n3; ++k) e3 += st[k];
        fprintf(f, "%le %le %le %le %le\n", e5[0], e5[1], e5[2], e3, e5[4]);
        fclose(f);
    }
    return TIS_OK;
}

int tis_read_last_frame(const char *coordinates, int n, double *x, double *y, double *z, int64_t *frames)
{
    if (!coordinates || n < 1 || !frames) return fail(TIS_ERR_ARG, "tis_read_last_frame: bad argument");
    *frames = 0;
    FILE *f = fopen(coordinates, "rb");
    if (!f) return fail(TIS_ERR_IO, "cannot open %s", coordinates);
    std::vector<double> buf(3 * ((size_t)n + 1));
    int64_t count = 0;
    while (fread(buf.data(), sizeof(double), buf.size(), f) == buf.size()) {
        ++count;
        if (x) memcpy(x, buf.data() + 1, sizeof(double) * n);
        if (y) memcpy(y, buf.data() + (n + 1) + 1, sizeof(double) * n);
        if (z) memcpy(z, buf.data() + 2 * (n + 1) + 1, sizeof(double) * n);
    }
    const bool partial = !feof(f) || ftell(f) % (long)(sizeof(double) * buf.size()) != 0;
    fclose(f);
    *frames = count;
    if (partial) return fail(TIS_ERR_FORMAT, "%s: trailing partial frame", coordinates);
    return TIS_OK;
}

namespace {

int64_t sys_i64(const tis_system *s, const char *name, int64_t def)
{
    const tis::Array *a = s->get(name);
    if (!a || a->count() < 1) return def;
    if (a->dtype == TIS_I64) return a->as<int64_t>()[0];
    if (a->dtype == TIS_I32) return a->as<int32_t>()[0];
    return (int64_t)a->as<double>()[0];
}

bool put_i32(FILE *f, int32_t v) { return fwrite(&v, 4, 1, f) == 1; }

}  // namespace

int tis_write_psf(const tis_system *s, const char *path)
{
    if (!s || !path) return fail(TIS_ERR_ARG, "tis_write_psf: bad argument");
    const int n = (int)sys_i64(s, "n_particles", -1), ntp = (int)sys_i64(s, "n_rna", -1);
    const tis::Array *type = s->get("type"), *kind = s->get("kind");
    if (n < 1 || ntp < 1 || ntp > n || !type || !kind || type->dtype != TIS_I32 || kind->dtype != TIS_I32 ||
        type->count() != n || kind->count() != n)
        return fail(TIS_ERR_ARG, "tis_write_psf: the system lacks n_particles, n_rna, type or kind");
    const int32_t *ty = type->as<int32_t>(), *kd = kind->as<int32_t>();
    // the nucleotide letter of bead i (1-based): its base bead's type (3 A, 4 G, 5 C, 6 U)
    auto letter = [&](int i) {
        const int b = 3 * (i / 3) + 1;  // 0-based index of the base bead of nucleotide i / 3 + 1
        const int t = b < ntp ? ty[b] : 0;
        return t == 3 ? 'A' : t == 4 ? 'G' : t == 5 ? 'C' : t == 6 ? 'U' : 'N';
    };
    FILE *f = fopen(path, "w");
    if (!f) return fail(TIS_ERR_IO, "cannot open %s", path);
    // the layout of the reference's topology exporter (analysis/make_ninfo/16SCD_ninfo.cpp:6563-6650)
    fprintf(f, "%8i !NATOM\n", n);
    for (int i = 1; i <= ntp; ++i) {
        const char c = letter(i);
        fprintf(f, "%8iR%c %4i      R%c", i, c, i / 3 + 1, c);
        if (i % 3 == 1) fprintf(f, "    S   S     %11.6f%14.4f", 0.0, 10.0);
        else if (i % 3 == 2) fprintf(f, "    %cb  B     %11.6f%14.4f", c, 0.0, 10.0);
        else fprintf(f, "    P   P     %11.6f%14.4f", -1.0, 10.0);
        fprintf(f, "           0\n");
    }
    for (int i = ntp + 1; i <= n; ++i) {
        const int k = kd[i - 1];  // part_key: 3 Mg, 4 Cl, 5 K
        const char *nm = k == 3 ? "Mg " : k == 4 ? "Cl " : "K  ";
        const char *r2 = k == 3 ? "Mg" : k == 4 ? "Cl" : "K ";
        const double q = k == 3 ? 2.0 : k == 4 ? -1.0 : 1.0;
        fprintf(f, "%8i%s%4i      %s    %s  %s    %11.6f%14.4f           0\n", i, nm, ntp / 3 + i - ntp + 1, r2, r2,
                r2, q, 10.0);
    }
    fprintf(f, "%8i !NBOND\n", ntp - 1);
    int col = 0;
    for (int i = 2; i <= ntp; ++i) {  // P-S, S-B of a nucleotide; S-P to the next one
        fprintf(f, "%8i%8i", i % 3 == 0 ? i - 2 : i - 1, i);
        if (++col == 4) {
            fprintf(f, "\n");
            col = 0;
        }
    }
    const bool ok = !ferror(f);
    fclose(f);
    return ok ? TIS_OK : fail(TIS_ERR_IO, "short write to %s", path);
}

int tis_write_cgpdb(const tis_system *s, const double *x, const double *y, const double *z, const char *path)
{
    if (!s || !path) return fail(TIS_ERR_ARG, "tis_write_cgpdb: bad argument");
    const int n = (int)sys_i64(s, "n_particles", -1), ntp = (int)sys_i64(s, "n_rna", -1);
    const int nbp = (int)sys_i64(s, "n_entries", -1);
    const tis::Array *type = s->get("type"), *kind = s->get("kind");
    if (n < 1 || ntp < 1 || ntp > n || nbp < 1 || !type || !kind || type->dtype != TIS_I32 ||
        kind->dtype != TIS_I32 || type->count() != n || kind->count() != n)
        return fail(TIS_ERR_ARG, "tis_write_cgpdb: the system lacks n_particles, n_rna, n_entries, type or kind");
    const double *c[3] = {x, y, z};
    const char *nm[3] = {"x", "y", "z"};
    for (int a = 0; a < 3; ++a)
        if (!c[a]) {  // the system's own (set-up) coordinates
            const tis::Array *arr = s->get(nm[a]);
            if (!arr || arr->dtype != TIS_F64 || arr->count() != n) return fail(TIS_ERR_ARG, "tis_write_cgpdb: no %s", nm[a]);
            c[a] = arr->as<double>();
        }
    const int32_t *ty = type->as<int32_t>(), *kd = kind->as<int32_t>();
    auto letter = [&](int i) {
        const int b = 3 * (i / 3) + 1;
        const int t = b < ntp ? ty[b] : 0;
        return t == 3 ? 'A' : t == 4 ? 'G' : t == 5 ? 'C' : t == 6 ? 'U' : 'N';
    };
    FILE *f = fopen(path, "w");
    if (!f) return fail(TIS_ERR_IO, "cannot open %s", path);
    // the layout of the reference's exporter (analysis/make_ninfo/16SCD_ninfo.cpp:6479-6561): its
    // counts are the PDB entries (N_amino = NBP_atom), entries plus ions (NB_atom), RNA beads
    // (NTP_atom), RNA bead pairs (NpTP_atom) and particles (NT_atom)
    fprintf(f, "RECORD   N_amino   %5i\n", nbp);
    fprintf(f, "RECORD   NBP_atom  %5i\n", nbp);
    fprintf(f, "RECORD   NB_atom   %5i\n", nbp + (n - ntp));
    fprintf(f, "RECORD   NTP_atom  %5i\n", ntp);
    fprintf(f, "RECORD   NpTP_atom %5i\n", ntp * (ntp + 1) / 2);
    fprintf(f, "RECORD   NT_atom   %5i\n", n);
    for (int i = 1; i <= ntp; ++i) {
        const char l = letter(i);
        if (i % 3 == 1) fprintf(f, "ATOM  %5i  S   R%c  A%4i", i, l, i / 3 + 1);
        else if (i % 3 == 2) fprintf(f, "ATOM  %5i  %cb  R%c  A%4i", i, l, l, i / 3 + 1);
        else fprintf(f, "ATOM  %5i  P   R%c  A%4i", i, l, i / 3 + 1);
        fprintf(f, "    %8.3f%8.3f%8.3f\n", c[0][i - 1], c[1][i - 1], c[2][i - 1]);
    }
    fprintf(f, "TER\n");
    for (int i = ntp + 1; i <= n; ++i) {
        const int k = kd[i - 1];
        const char *nmr = k == 3 ? "MG    MG" : k == 4 ? " Cl   Cl" : " K    K ";
        fprintf(f, "ATOM  %5i %s B%4i    %8.3f%8.3f%8.3f\n", i, nmr, i, c[0][i - 1], c[1][i - 1], c[2][i - 1]);
    }
    fprintf(f, "TER\n");
    const bool ok = !ferror(f);
    fclose(f);
    return ok ? TIS_OK : fail(TIS_ERR_IO, "short write to %s", path);
}

}  // extern "C"

namespace {

// the arrays of a loaded system the topology exporter reads
struct SysView {
    const tis_system *s;
    template <class T>
    const T *arr(const char *name, int dtype, int64_t *count) const
    {
        const tis::Array *a = s->get(name);
        if (!a || a->dtype != dtype) return nullptr;
        *count = a->count();
        return a->as<T>();
    }
};

constexpr double kPi = 3.14159265358979323846264338328;

// dihedral angle i1-i2-i3-i4 (0-based beads; -1: the origin, as the exporter reads
// its unused bead 0), atan2 of the triple product over the normals' dot product
double dihedral_host(const double *x, const double *y, const double *z, int i1, int i2, int i3, int i4)
{
    auto P = [&](int i, int c) { return i < 0 ? 0.0 : (c == 0 ? x[i] : c == 1 ? y[i] : z[i]); };
    double v1[3], v2[3], v3[3];
    for (int c = 0; c < 3; ++c) {
        v1[c] = P(i2, c) - P(i1, c);
        v2[c] = P(i3, c) - P(i2, c);
        v3[c] = P(i4, c) - P(i3, c);
    }
    const double m[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
    const double n[3] = {v2[1] * v3[2] - v2[2] * v3[1], v2[2] * v3[0] - v2[0] * v3[2], v2[0] * v3[1] - v2[1] * v3[0]};
    const double l = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
    return atan2((v1[0] * n[0] + v1[1] * n[1] + v1[2] * n[2]) * l, m[0] * n[0] + m[1] * n[1] + m[2] * n[2]);
}

// the value of a native periodic coordinate nat imaged to within pi of psi
double image_near(double psi, double nat)
{
    if (fabs(psi - nat) <= kPi) return nat;
    return psi - nat > kPi ? nat + 2.0 * kPi : nat - 2.0 * kPi;
}

}  // namespace

extern "C" {

int tis_write_ninfo(const tis_system *s, const char *path)
{
    if (!s || !path) return fail(TIS_ERR_ARG, "tis_write_ninfo: bad argument");
    const SysView V{s};
    int64_t ne = 0, nb = 0, n3 = 0, n2 = 0, nh = 0, c = 0, nx = 0, nst = 0;
    const int32_t *ea0 = V.arr<int32_t>("entry_a0", TIS_I32, &ne), *ea1 = V.arr<int32_t>("entry_a1", TIS_I32, &c),
                  *ecode = V.arr<int32_t>("entry_code", TIS_I32, &c);
    const int32_t *bk = V.arr<int32_t>("bt_kind", TIS_I32, &nb), *ba = V.arr<int32_t>("bt_a", TIS_I32, &c),
                  *bb = V.arr<int32_t>("bt_b", TIS_I32, &c), *bc = V.arr<int32_t>("bt_c", TIS_I32, &c);
    const double *bk0 = V.arr<double>("bt_k0", TIS_F64, &c), *bx0 = V.arr<double>("bt_x0", TIS_F64, &c);
    const int32_t *i3 = V.arr<int32_t>("st3_idx", TIS_I32, &n3), *site = V.arr<int32_t>("st3_site", TIS_I32, &c),
                  *exc = V.arr<int32_t>("st_excess", TIS_I32, &nst);
    const double *nat3 = V.arr<double>("st3_native", TIS_F64, &c), *E3 = V.arr<double>("st3_E", TIS_F64, &c);
    const int32_t *i2 = V.arr<int32_t>("st2_idx", TIS_I32, &n2), *e2 = V.arr<int32_t>("st2_entry_i", TIS_I32, &c);
    const double *r02 = V.arr<double>("st2_r0", TIS_F64, &c), *E2 = V.arr<double>("st2_E", TIS_F64, &c);
    const int32_t *ih = V.arr<int32_t>("hb_idx", TIS_I32, &nh), *dode = V.arr<int32_t>("hb_dode", TIS_I32, &c);
    const double *nath = V.arr<double>("hb_native", TIS_F64, &c), *Eh = V.arr<double>("hb_E", TIS_F64, &c);
    const double *x = V.arr<double>("x", TIS_F64, &nx), *y = V.arr<double>("y", TIS_F64, &c),
                 *z = V.arr<double>("z", TIS_F64, &c);
    if (!ea0 || !ea1 || !ecode || !bk || !ba || !bb || !bc || !bk0 || !bx0 || !i3 || !site || !exc || !nat3 || !E3 ||
        !i2 || !e2 || !r02 || !E2 || !ih || !dode || !nath || !Eh || !x || !y || !z)
        return fail(TIS_ERR_ARG, "tis_write_ninfo: the system lacks its topology arrays (a loaded system has them)");
    n3 /= 6;
    n2 /= 7;
    nh /= 6;
    // bond and angle parameters of the loaded topology, keyed by their beads
    std::map<std::pair<int, int>, std::pair<double, double>> bonds;
    std::map<std::array<int, 3>, std::pair<double, double>> angles;
    for (int64_t t = 0; t < nb; ++t) {
        if (bk[t] == 0) bonds[{std::min(ba[t], bb[t]), std::max(ba[t], bb[t])}] = {bk0[t], bx0[t]};
        else angles[{bb[t], std::min(ba[t], bc[t]), std::max(ba[t], bc[t])}] = {bk0[t], bx0[t]};
    }
    auto bond = [&](int a, int b, std::pair<double, double> *kv) {
        auto it = bonds.find({std::min(a, b), std::max(a, b)});
        if (it == bonds.end()) return false;
        *kv = it->second;
        return true;
    };
    auto angle = [&](int a, int m, int b, std::pair<double, double> *kv) {
        auto it = angles.find({m, std::min(a, b), std::max(a, b)});
        if (it == angles.end()) return false;
        *kv = it->second;
        return true;
    };
    FILE *f = fopen(path, "w");
    if (!f) return fail(TIS_ERR_IO, "cannot open %s", path);
    bool missing = false;
    // the exporter's records (analysis/make_ninfo/16SCD_ninfo.cpp): bonds and angles
    // (:6083-6250), then stacks (:5840-5997), then H-bonds (:6000-6080); bead
    // numbers 1-based, angles in degrees
    int ibd = 0, iangl = 0;
    auto put_bond = [&](int a, int b, const char *tag) {
        std::pair<double, double> kv;
        if (!bond(a, b, &kv)) {
            missing = true;
            return;
        }
        ++ibd;
        fprintf(f, "bond %6i %2i %2i %4i %4i %4i %4i %12.4f %3.1f %3.1f %12.4f %s\n", ibd, 1, 1, a + 1, b + 1, a + 1,
                b + 1, kv.second, 1.0, 1.0, kv.first, tag);
    };
    auto put_angle = [&](int a, int m, int b, const char *tag) {
        std::pair<double, double> kv;
        if (!angle(a, m, b, &kv)) {
            missing = true;
            return;
        }
        ++iangl;
        fprintf(f, "angl %6i %2i %2i %4i %4i %4i %4i %4i %4i", iangl, 1, 1, a + 1, m + 1, b + 1, a + 1, m + 1, b + 1);
        fprintf(f, "%12.4f %3.1f %3.1f %12.4f %s\n", kv.second / kPi * 180.0, 1.0, 1.0, kv.first, tag);
    };
    const int NBP = (int)ne;
    for (int e = 1; e <= NBP; e += 2) {  // sugar-base bond, base angles of each nucleotide
        const char b = (char)ecode[e - 1];
        if (b != 'A' && b != 'C' && b != 'G' && b != 'U') continue;
        const int si = ea0[e - 1], bi = ea1[e - 1];
        char tag[8];
        snprintf(tag, sizeof tag, "S%c", b);
        put_bond(si, bi, tag);
        if (e < NBP) {
            snprintf(tag, sizeof tag, "%cSP", b);
            put_angle(bi, si, ea0[e], tag);
        }
        if (e > 1) {
            snprintf(tag, sizeof tag, "PS%c", b);
            put_angle(ea0[e - 2], si, bi, tag);
        }
    }
    for (int e = 2; e <= NBP; e += 2) {  // sugar-phosphate bonds, P-S-P angles
        const int pi_ = ea0[e - 1], si = ea0[e - 2];
        put_bond(si, pi_, "SP");
        if (e > 2) put_angle(ea0[e - 3], si, pi_, "PSP");
    }
    for (int e = 3; e <= NBP; e += 2) {  // phosphate-sugar bonds, S-P-S angles
        const int si = ea0[e - 1], pj = ea0[e - 2], sk = ea0[e - 3];
        put_bond(pj, si, "PS");
        put_angle(sk, pj, si, "SPS");
    }
    // tertiary stacks: distance, two angles, three dihedrals at their natives
    int it = 0, itang = 0, itdih = 0;
    for (int64_t k = 0; k < n3; ++k) {
        const int *q = i3 + 6 * k;  // k10 k11 k12 k20 k21 k22
        const double *nv = nat3 + 6 * k;
        const int s0 = site[2 * k], s1 = site[2 * k + 1];
        const int ii = (s0 >= 1 && s0 <= nst && exc[s0 - 1] == 1) ? 2 : 1;
        const int jj = (s1 >= 1 && s1 <= nst && exc[s1 - 1] == 1) ? 2 : 1;
        ++it;
        fprintf(f, "tbs-dist %6i %2i %2i %4i %4i %4i %4i %9.3f %7.2f 5.0 %3i %3i\n", it, 1, 1, q[1] + 1, q[4] + 1,
                q[1] + 1, q[4] + 1, E3[k], nv[0], ii, jj);
        const int ang[2][3] = {{q[0], q[1], q[4]}, {q[3], q[4], q[1]}};
        for (int a = 0; a < 2; ++a) {
            ++itang;
            fprintf(f, "tbs-angl %6i %6i %2i %2i %4i %4i %4i %4i %4i %4i", it, itang, 1, 1, ang[a][0] + 1,
                    ang[a][1] + 1, ang[a][2] + 1, ang[a][0] + 1, ang[a][1] + 1, ang[a][2] + 1);
            fprintf(f, " %7.2f %3.1f\n", nv[1 + a] / kPi * 180.0, 1.5);
        }
        const int dih[3][4] = {{q[0], q[1], q[4], q[3]}, {q[4], q[1], q[0], q[2]}, {q[1], q[4], q[3], q[5]}};
        for (int a = 0; a < 3; ++a) {
            ++itdih;
            fprintf(f, "tbs-dihd %6i %6i %2i %2i", it, itdih, 1, 1);
            for (int r = 0; r < 2; ++r)
                for (int u = 0; u < 4; ++u) fprintf(f, " %4i", dih[a][u] + 1);
            fprintf(f, " %7.2f %4.2f\n", nv[3 + a] / kPi * 180.0, 0.15);
        }
    }
    // secondary stacks: distance, and the two backbone dihedrals imaged near their
    // fixed natives (-2.58684, 3.07135) from the loaded positions
    int is = 0, isdih = 0;
    for (int64_t k = 0; k < n2; ++k) {
        const int *q = i2 + 7 * k;  // k_10 k00 k01 k10 k20 k21 k30
        const int e = e2[k];
        const char l0 = e >= 1 && e <= NBP ? (char)ecode[e - 1] : 'N';
        const char l1 = e + 2 >= 1 && e + 2 <= NBP ? (char)ecode[e + 1] : 'N';
        const double psi1 = dihedral_host(x, y, z, q[0], q[1], q[3], q[4]);
        const double psi2 = dihedral_host(x, y, z, q[6], q[4], q[3], q[1]);
        const double p10 = image_near(psi1, -2.58684), p20 = image_near(psi2, 3.07135);
        ++is;
        fprintf(f, "bs-dist %6i %2i %2i %4i %4i %4i %4i %9.3f %7.2f 1.40 %c-%c\n", is, 1, 1, q[2] + 1, q[5] + 1,
                q[2] + 1, q[5] + 1, E2[k], r02[k], l0, l1);
        const int dih[2][4] = {{q[0], q[1], q[3], q[4]}, {q[1], q[3], q[4], q[6]}};
        const double nat[2] = {p10, p20};
        const char *tag[2] = {"PSPS", "SPSP"};
        for (int a = 0; a < 2; ++a) {
            ++isdih;
            fprintf(f, "bs-dihd %6i %6i %2i %2i", is, isdih, 1, 1);
            for (int r = 0; r < 2; ++r)
                for (int u = 0; u < 4; ++u) fprintf(f, " %4i", dih[a][u] + 1);
            fprintf(f, " %7.2f %3.1f %s\n", nat[a] / kPi * 180.0, 4.0, tag[a]);
        }
    }
    // hydrogen-bond candidates: distance (T tertiary, S secondary), two angles,
    // three dihedrals at their natives
    int ihb = 0, ihang = 0, ihdih = 0;
    for (int64_t k = 0; k < nh; ++k) {
        const int *q = ih + 6 * k;  // k10 k11 k12 k20 k21 k22
        const double *nv = nath + 6 * k;
        ++ihb;
        fprintf(f, "hb-dist %6i %2i %2i %4i %4i %4i %4i %9.3f %7.2f 5.0 %c\n", ihb, 1, 1, q[1] + 1, q[4] + 1,
                q[1] + 1, q[4] + 1, Eh[k], nv[0], dode[k] ? 'T' : 'S');
        const int ang[2][3] = {{q[0], q[1], q[4]}, {q[3], q[4], q[1]}};
        for (int a = 0; a < 2; ++a) {
            ++ihang;
            fprintf(f, "hb-angl %6i %6i %2i %2i %4i %4i %4i %4i %4i %4i", ihb, ihang, 1, 1, ang[a][0] + 1,
                    ang[a][1] + 1, ang[a][2] + 1, ang[a][0] + 1, ang[a][1] + 1, ang[a][2] + 1);
            fprintf(f, " %7.2f %3.1f\n", nv[1 + a] / kPi * 180.0, 1.5);
        }
        const int dih[3][4] = {{q[0], q[1], q[4], q[3]}, {q[4], q[1], q[0], q[2]}, {q[1], q[4], q[3], q[5]}};
        for (int a = 0; a < 3; ++a) {
            ++ihdih;
            fprintf(f, "hb-dihd %6i %6i %2i %2i", ihb, ihdih, 1, 1);
            for (int r = 0; r < 2; ++r)
                for (int u = 0; u < 4; ++u) fprintf(f, " %4i", dih[a][u] + 1);
            fprintf(f, " %7.2f %4.2f\n", nv[3 + a] / kPi * 180.0, 0.15);
        }
    }
    const bool ok = !ferror(f);
    fclose(f);
    if (missing) return fail(TIS_ERR_FORMAT, "tis_write_ninfo: a bond or angle of the chain is not in the topology");
    return ok ? TIS_OK : fail(TIS_ERR_IO, "short write to %s", path);
}

int tis_write_dcd(tis_handle *h, int replica, const char *path, int32_t nsavc, double delta)
{
    if (!h || !path || nsavc < 1) return fail(TIS_ERR_ARG, "tis_write_dcd: bad argument");
    int n = 0, rc;
    if ((rc = tis_replica_size(h, replica, &n))) return rc;
    std::vector<double> x(n), y(n), z(n);
    if ((rc = tis_get_state(h, replica, x.data(), y.data(), z.data(), nullptr, nullptr, nullptr, nullptr, nullptr,
                            nullptr)))
        return rc;
    FILE *f = fopen(path, "r+b");
    int32_t nset = 0;
    if (f) {
        char head[8];
        if (fread(head, 1, 8, f) != 8 || memcmp(head + 4, "CORD", 4) != 0 || fread(&nset, 4, 1, f) != 1) {
            fclose(f);
            return fail(TIS_ERR_FORMAT, "%s: not a DCD file written here", path);
        }
        int32_t natom = 0;  // record 3, after the 84-byte control record and the title record
        int32_t tlen = 0;
        if (fseek(f, 4 + 84 + 4, SEEK_SET) || fread(&tlen, 4, 1, f) != 1 || fseek(f, tlen + 4 + 4, SEEK_CUR) ||
            fread(&natom, 4, 1, f) != 1 || natom != n) {
            fclose(f);
            return fail(TIS_ERR_FORMAT, "%s: %d atoms, the replica has %d", path, natom, n);
        }
        fseek(f, 0, SEEK_END);
    } else {
        f = fopen(path, "w+b");
        if (!f) return fail(TIS_ERR_IO, "cannot open %s", path);
        // CHARMM/NAMD DCD: control record (NSET, ISTART, NSAVC, NSTEP, ..., DELTA, ..., version 24)
        int32_t ic[20] = {0};
        ic[1] = nsavc;
        ic[2] = nsavc;
        const float dt = (float)delta;
        memcpy(&ic[9], &dt, 4);
        ic[19] = 24;
        bool ok = put_i32(f, 84) && fwrite("CORD", 1, 4, f) == 4 && fwrite(ic, 4, 20, f) == 20 && put_i32(f, 84);
        char title[2][80];
        memset(title, ' ', sizeof title);
        const char *t0 = "REMARKS TIS-RNA Langevin engine (GB300)";
        memcpy(title[0], t0, strlen(t0));
        char t1[81];
        snprintf(t1, sizeof t1, "REMARKS replica %d, a frame every %d steps", replica, nsavc);
        memcpy(title[1], t1, strlen(t1));
        ok = ok && put_i32(f, 4 + 160) && put_i32(f, 2) && fwrite(title, 1, 160, f) == 160 && put_i32(f, 4 + 160);
        ok = ok && put_i32(f, 4) && put_i32(f, n) && put_i32(f, 4);
        if (!ok) {
            fclose(f);
            return fail(TIS_ERR_IO, "short write to %s", path);
        }
    }
    std::vector<float> buf(n);
    bool ok = true;
    for (const std::vector<double> *a : {&x, &y, &z}) {
        for (int i = 0; i < n; ++i) buf[i] = (float)(*a)[i];
        ok = ok && put_i32(f, 4 * n) && fwrite(buf.data(), 4, n, f) == (size_t)n && put_i32(f, 4 * n);
    }
    ++nset;
    const int32_t nstep = nset * nsavc;
    ok = ok && fseek(f, 8, SEEK_SET) == 0 && put_i32(f, nset) && fseek(f, 8 + 12, SEEK_SET) == 0 && put_i32(f, nstep);
    fclose(f);
    return ok ? TIS_OK : fail(TIS_ERR_IO, "short write to %s", path);
}

}  // extern "C"
