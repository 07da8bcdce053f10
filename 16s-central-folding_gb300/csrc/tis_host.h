// Host-side internals shared by the system, loader and engine translation units.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "../../include/tis_gpu.h"

namespace tis {

// Records the error text for tis_last_error and returns the code.
int fail(int code, const char *fmt, ...);
void clear_error();

struct Array {
    int dtype = TIS_F64;
    std::vector<char> bytes;
    int64_t count() const { return (int64_t)bytes.size() / (dtype == TIS_I32 ? 4 : 8); }
    template <class T>
    const T *as() const { return reinterpret_cast<const T *>(bytes.data()); }
};

}  // namespace tis

struct tis_system {
    std::map<std::string, tis::Array> arrays;

    void set_f64(const std::string &n, const std::vector<double> &v);
    void set_i32(const std::string &n, const std::vector<int32_t> &v);
    void set_i64(const std::string &n, int64_t v);
    void set_scalar(const std::string &n, double v);
    bool has(const std::string &n) const { return arrays.count(n) != 0; }
    const tis::Array *get(const std::string &n) const
    {
        auto it = arrays.find(n);
        return it == arrays.end() ? nullptr : &it->second;
    }
};
