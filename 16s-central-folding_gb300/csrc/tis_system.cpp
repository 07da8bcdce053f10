// tis_system: a named set of arrays holding one replica's topology and state.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "tis_device.cuh"
#include "tis_host.h"

namespace tis {

static thread_local char g_err[1024] = {0};

int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

void clear_error() { g_err[0] = 0; }

}  // namespace tis

void tis_system::set_f64(const std::string &n, const std::vector<double> &v)
{
    tis::Array a;
    a.dtype = TIS_F64;
    a.bytes.resize(v.size() * 8);
    if (!v.empty()) memcpy(a.bytes.data(), v.data(), a.bytes.size());
    arrays[n] = std::move(a);
}

void tis_system::set_i32(const std::string &n, const std::vector<int32_t> &v)
{
    tis::Array a;
    a.dtype = TIS_I32;
    a.bytes.resize(v.size() * 4);
    if (!v.empty()) memcpy(a.bytes.data(), v.data(), a.bytes.size());
    arrays[n] = std::move(a);
}

void tis_system::set_i64(const std::string &n, int64_t v)
{
    tis::Array a;
    a.dtype = TIS_I64;
    a.bytes.resize(8);
    memcpy(a.bytes.data(), &v, 8);
    arrays[n] = std::move(a);
}

void tis_system::set_scalar(const std::string &n, double v) { set_f64(n, std::vector<double>{v}); }

extern "C" {

int tis_last_error(char *buf, size_t n)
{
    if (!buf || n == 0) return TIS_ERR_ARG;
    snprintf(buf, n, "%s", tis::g_err);
    return TIS_OK;
}

int tis_system_new(tis_system **out)
{
    if (!out) return tis::fail(TIS_ERR_ARG, "tis_system_new: null output");
    *out = new tis_system();
    return TIS_OK;
}

int tis_system_set(tis_system *s, const char *name, int dtype, const void *data, int64_t count)
{
    if (!s || !name || count < 0 || (count > 0 && !data)) return tis::fail(TIS_ERR_ARG, "tis_system_set: bad argument");
    if (dtype != TIS_F64 && dtype != TIS_I32 && dtype != TIS_I64)
        return tis::fail(TIS_ERR_ARG, "tis_system_set(%s): unknown dtype %d", name, dtype);
    tis::Array a;
    a.dtype = dtype;
    a.bytes.resize((size_t)count * (dtype == TIS_I32 ? 4 : 8));
    if (count) memcpy(a.bytes.data(), data, a.bytes.size());
    s->arrays[name] = std::move(a);
    return TIS_OK;
}

int tis_system_get(const tis_system *s, const char *name, int *dtype, const void **data, int64_t *count)
{
    if (!s || !name) return tis::fail(TIS_ERR_ARG, "tis_system_get: bad argument");
    const tis::Array *a = s->get(name);
    if (!a) return tis::fail(TIS_ERR_ARG, "tis_system_get: no array '%s'", name);
    if (dtype) *dtype = a->dtype;
    if (data) *data = a->bytes.data();
    if (count) *count = a->count();
    return TIS_OK;
}

int tis_system_count(const tis_system *s, int *n)
{
    if (!s || !n) return tis::fail(TIS_ERR_ARG, "tis_system_count: bad argument");
    *n = (int)s->arrays.size();
    return TIS_OK;
}

int tis_system_name(const tis_system *s, int i, const char **name)
{
    if (!s || !name || i < 0 || i >= (int)s->arrays.size()) return tis::fail(TIS_ERR_ARG, "tis_system_name: bad index");
    auto it = s->arrays.begin();
    std::advance(it, i);
    *name = it->first.c_str();
    return TIS_OK;
}

int tis_system_destroy(tis_system *s)
{
    delete s;
    return TIS_OK;
}

int tis_rand_stream(uint64_t seed, uint64_t first, int64_t n, int32_t *out)
{
    if (n < 0 || (n > 0 && !out)) return tis::fail(TIS_ERR_ARG, "tis_rand_stream: bad argument");
    for (int64_t k = 0; k < n; ++k) out[k] = (int32_t)tis::rand_value(seed, first + (uint64_t)k);
    return TIS_OK;
}

}  // extern "C"
