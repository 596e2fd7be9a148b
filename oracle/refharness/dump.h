/* dump.h -- tiny named-array container used by the reference harnesses:
 * records of {char name[32]; char dtype[8]; uint64 count; data}. */
#ifndef DSIM_REFHARNESS_DUMP_H
#define DSIM_REFHARNESS_DUMP_H
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <string>
#include <map>
static inline void dump_rec(FILE* f, const char* name, const char* dtype, const void* data,
                            uint64_t count, size_t elem) {
    char n[32] = {0}, d[8] = {0};
    strncpy(n, name, 31); strncpy(d, dtype, 7);
    fwrite(n, 1, 32, f); fwrite(d, 1, 8, f); fwrite(&count, 8, 1, f);
    if (count) fwrite(data, elem, count, f);
}
static inline std::map<std::string, std::string> parse_kv(int argc, char** argv) {
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; i++) {
        const char* eq = strchr(argv[i], '=');
        if (eq) kv[std::string(argv[i], eq - argv[i])] = std::string(eq + 1);
    }
    return kv;
}
static inline double kvd(std::map<std::string, std::string>& kv, const char* k, double def) {
    auto it = kv.find(k);
    return it == kv.end() ? def : atof(it->second.c_str());
}
static inline double now_ms() {
    struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}
#endif
