// The reference's output files (E:6276-6312) and its restart read (E:6181-6211).
#include <cstdio>
#include <cstring>
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
