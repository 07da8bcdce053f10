/* TEST INFRASTRUCTURE: reader/writer for the "TISB" record files exchanged
 * between the reference harness, the C oracle and the Python tests.
 *
 * Layout: 8-byte magic "TISB0001", then records
 *   char name[32] (NUL padded) | char dtype[4] ("f8", "i4", "i8") | int64 count | data
 * all little-endian, data packed. */
#ifndef TIS_TISB_IO_H
#define TIS_TISB_IO_H
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static inline FILE *tisb_open_write(const char *path)
{
    FILE *f = fopen(path, "wb");
    if (f) fwrite("TISB0001", 1, 8, f);
    return f;
}

static inline void tisb_put(FILE *f, const char *name, const char *dtype, const void *data, int64_t count)
{
    char nm[32] = {0}, dt[4] = {0};
    size_t es = (dtype[0] == 'f' || dtype[1] == '8') ? 8 : 4;
    strncpy(nm, name, 31);
    strncpy(dt, dtype, 3);
    fwrite(nm, 1, 32, f);
    fwrite(dt, 1, 4, f);
    fwrite(&count, 8, 1, f);
    if (count > 0) fwrite(data, es, (size_t)count, f);
}

static inline void tisb_put_f8(FILE *f, const char *name, const double *d, int64_t n) { tisb_put(f, name, "f8", d, n); }
static inline void tisb_put_i4(FILE *f, const char *name, const int32_t *d, int64_t n) { tisb_put(f, name, "i4", d, n); }
static inline void tisb_put_scalar_f8(FILE *f, const char *name, double v) { tisb_put(f, name, "f8", &v, 1); }
static inline void tisb_put_scalar_i8(FILE *f, const char *name, int64_t v) { tisb_put(f, name, "i8", &v, 1); }

#endif
