/*
 * harness_io.h -- key/value record files used to drive the reference's own
 * C++ classes from the test suite (TEST INFRASTRUCTURE ONLY).
 *
 * Record: int32 name length, name bytes, int64 count, count float64 values.
 * Integer quantities travel as float64.  Node fields travel in U order
 * (u = k*ni*nj + j*ni + i); particles as a 7 x n block x,y,z,vx,vy,vz,mpw.
 */
#ifndef HARNESS_IO_H
#define HARNESS_IO_H
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <vector>

typedef std::map<std::string, std::vector<double>> KV;

static inline KV kv_read(const char *path) {
    KV kv;
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    for (;;) {
        int32_t len;
        if (fread(&len, 4, 1, f) != 1) break;
        std::string name(len, ' ');
        if (fread(&name[0], 1, len, f) != (size_t)len) exit(3);
        int64_t cnt;
        if (fread(&cnt, 8, 1, f) != 1) exit(3);
        std::vector<double> v(cnt);
        if (cnt && fread(v.data(), 8, cnt, f) != (size_t)cnt) exit(3);
        kv[name] = v;
    }
    fclose(f);
    return kv;
}

static inline void kv_write(const char *path, const KV &kv) {
    FILE *f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path); exit(2); }
    for (auto &it : kv) {
        int32_t len = (int32_t)it.first.size();
        fwrite(&len, 4, 1, f);
        fwrite(it.first.data(), 1, len, f);
        int64_t cnt = (int64_t)it.second.size();
        fwrite(&cnt, 8, 1, f);
        if (cnt) fwrite(it.second.data(), 8, cnt, f);
    }
    fclose(f);
}

static inline const std::vector<double> &kv_get(const KV &kv, const char *k) {
    auto it = kv.find(k);
    if (it == kv.end()) { fprintf(stderr, "missing key %s\n", k); exit(4); }
    return it->second;
}
static inline double kv_s(const KV &kv, const char *k) { return kv_get(kv, k).at(0); }
static inline bool kv_has(const KV &kv, const char *k) { return kv.count(k) > 0; }

/* Node-field helpers over the reference's Field_ (data[i][j][k] access). */
template <class F>
static inline void field_in(F &f, const std::vector<double> &v, int ni, int nj, int nk) {
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) f[i][j][k] = v.at((size_t)k * ni * nj + (size_t)j * ni + i);
}
template <class F>
static inline std::vector<double> field_out(F &f, int ni, int nj, int nk) {
    std::vector<double> v((size_t)ni * nj * nk);
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) v[(size_t)k * ni * nj + (size_t)j * ni + i] = f[i][j][k];
    return v;
}
template <class F>
static inline void field3_in(F &f, const std::vector<double> &v, int ni, int nj, int nk) {
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                for (int c = 0; c < 3; c++)
                    f[i][j][k][c] = v.at(3 * ((size_t)k * ni * nj + (size_t)j * ni + i) + c);
}
template <class F>
static inline std::vector<double> field3_out(F &f, int ni, int nj, int nk) {
    std::vector<double> v(3 * (size_t)ni * nj * nk);
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                for (int c = 0; c < 3; c++)
                    v[3 * ((size_t)k * ni * nj + (size_t)j * ni + i) + c] = f[i][j][k][c];
    return v;
}
#endif
