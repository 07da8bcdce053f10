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

}  // extern "C"
