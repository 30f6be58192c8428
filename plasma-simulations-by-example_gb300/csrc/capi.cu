/*
 * capi.cu -- the extern "C" boundary of libespic (declared in include/espic.h).
 * Owns the device memory of a World, orders all of its work on one CUDA
 * stream and turns device error flags and CUDA errors into int status codes.
 * No C++ exception crosses this boundary.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "espic.h"
#include "espic_world.h"

using namespace espic;

struct espic_world {
    World w;
};

static thread_local std::string g_last_error;

static int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return fail(ESPIC_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define CHECK_LAUNCH()                                                                                      \
    do {                                                                                                    \
        cudaError_t e_ = cudaGetLastError();                                                                \
        if (e_ != cudaSuccess) return fail(ESPIC_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e_));    \
    } while (0)

#define WORLD(h)                                                        \
    if (!(h)) return fail(ESPIC_ERR_ARG, "null world handle");          \
    World &w = (h)->w;                                                  \
    if (cudaSetDevice(w.device) != cudaSuccess) return fail(ESPIC_ERR_CUDA, "cudaSetDevice failed")

#define SPECIES(sp)                                                                 \
    if ((sp) < 0 || (sp) >= (int)w.species.size())                                  \
        return fail(ESPIC_ERR_ARG, "species id %d out of range", (int)(sp));         \
    Species &s = *w.species[(sp)]

/* lets other translation units of the library report errors through
 * espic_last_error */
int espic_internal_fail(int code, const char *msg) { return fail(code, "%s", msg); }

extern "C" int espic_last_error(char *buf, int len) {
    if (!buf || len <= 0) return ESPIC_ERR_ARG;
    snprintf(buf, (size_t)len, "%s", g_last_error.c_str());
    return ESPIC_OK;
}

template <class T>
static int dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(ESPIC_ERR_CUDA, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
    }
    return ESPIC_OK;
}

/* device error flags -> status (clears them) */
static int take_device_errors(World &w) {
    int bits = 0;
    CK(cudaMemcpyAsync(&bits, w.d_err, sizeof(int), cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    if (bits) CK(cudaMemsetAsync(w.d_err, 0, sizeof(int), w.stream));
    if (bits & DERR_CAPACITY) return fail(ESPIC_ERR_CAPACITY, "particle capacity exceeded; particles not added");
    if (bits & DERR_NONFINITE) return fail(ESPIC_ERR_NONFINITE, "non-finite value in the step");
    if (bits & DERR_FIXED_RANGE) return fail(ESPIC_ERR_FIXED, "weight outside the fixed-point range");
    if (bits & DERR_TIMEOUT) return fail(ESPIC_ERR_CUDA, "a bounded wait on a bulk copy timed out");
    if (bits & DERR_SORT) return fail(ESPIC_ERR_CUDA, "the cell sort lost track of a particle");
    if (bits & DERR_DSMC)
        return fail(ESPIC_ERR_ARG, "DSMC: a particle outside the domain, or the replayed uniforms ran out");
    if (bits & DERR_NEUTRAL)
        return fail(ESPIC_ERR_ARG, "moments / MCC: a particle outside the grid, a non-finite moment, or a "
                                   "replayed uniform out of range");
    return ESPIC_OK;
}

/* ---- per-phase event timing ---- */
static void prof_collect(World &w) {
    if (w.ranges.empty()) return;
    cudaStreamSynchronize(w.stream);
    for (auto &r : w.ranges) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            w.prof_ms[r.phase] += ms;
            w.prof_n[r.phase] += 1;
        }
        w.ev_pool.push_back(r.a);
        w.ev_pool.push_back(r.b);
    }
    w.ranges.clear();
}

static cudaEvent_t prof_event(World &w) {
    if (w.ev_pool.empty()) {
        if (w.ranges.size() > 2048) prof_collect(w);
    }
    if (!w.ev_pool.empty()) {
        cudaEvent_t e = w.ev_pool.back();
        w.ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

struct PhaseScope {
    World &w;
    int phase;
    cudaEvent_t a = nullptr;
    PhaseScope(World &w_, int p) : w(w_), phase(p) {
        if (w.prof) {
            a = prof_event(w);
            cudaEventRecord(a, w.stream);
        }
    }
    ~PhaseScope() {
        if (w.prof && a) {
            cudaEvent_t b = prof_event(w);
            cudaEventRecord(b, w.stream);
            w.ranges.push_back({phase, a, b});
        }
    }
};

static void free_species(Species *s) {
    if (!s) return;
    void *ptrs[] = {s->P, s->cell, s->cell2, s->off, s->off2, s->vel, s->vel2, s->sort_count, s->deadmask,
                    s->tiledead, s->tilepre, s->holes, s->d_count, s->acc, s->den, s->den_ave, s->d_dsmc,
                    s->dsmc_cell, s->dsmc_rank, s->dsmc_perm, s->dsmc_count, s->dsmc_start, s->dsmc_bsum,
                    s->mom, s->mom_scale, s->gvel, s->gtemp, s->mpc, s->mom_acc, s->mom_bound, s->mcc_ncol,
                    s->ch4_settled, s->ch4_bounces, s->seg, s->ch4_cnt, s->ionize_cnt, s->dsum};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete s;
}

static void free_world(World &w) {
    for (Species *s : w.species) free_species(s);
    w.species.clear();
    void *ptrs[] = {w.phi, w.rho, w.vol, w.ivol, w.ef, w.ef4, w.pe_part, w.phi_ef, w.obj, w.target, w.d_err, w.d_status, w.d_partials,
                    w.d_small, w.d_u, w.d_stage, w.d_blockcnt, w.pcg_buf, w.phi_prev};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (w.h_small) cudaFreeHost(w.h_small);
    for (auto &sn : w.snap) {
        if (sn.copied) cudaEventSynchronize(sn.copied);
        if (sn.dev) cudaFree(sn.dev);
        if (sn.host) cudaFreeHost(sn.host);
        if (sn.packed) cudaEventDestroy(sn.packed);
        if (sn.copied) cudaEventDestroy(sn.copied);
    }
    if (w.snap_stream) cudaStreamDestroy(w.snap_stream);
    if (w.stream) cudaStreamSynchronize(w.stream);
    for (auto &r : w.ranges) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (cudaEvent_t e : w.ev_pool) cudaEventDestroy(e);
    if (w.stream) cudaStreamDestroy(w.stream);
}

extern "C" int espic_world_create(int ni, int nj, int nk, const double x0[3], const double xm[3],
                                  espic_world **out) {
    if (!out || !x0 || !xm) return fail(ESPIC_ERR_ARG, "null argument");
    *out = nullptr;
    if (ni < 3 || nj < 3 || nk < 3) return fail(ESPIC_ERR_ARG, "need at least 3 nodes per axis");
    for (int d = 0; d < 3; d++)
        if (!(xm[d] > x0[d])) return fail(ESPIC_ERR_ARG, "xm must exceed x0 on every axis");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(ESPIC_ERR_CUDA, "no CUDA device: libespic has no CPU path");
    espic_world *h = new espic_world();
    World &w = h->w;
    int rc = ESPIC_OK;
    cudaGetDevice(&w.device);
    cudaDeviceGetAttribute(&w.sm_count, cudaDevAttrMultiProcessorCount, w.device);
    w.g.ni = ni;
    w.g.nj = nj;
    w.g.nk = nk;
    int nn3[3] = {ni, nj, nk};
    for (int d = 0; d < 3; d++) {
        w.g.x0[d] = x0[d];
        w.g.xm[d] = xm[d];
        w.g.dh[d] = (xm[d] - x0[d]) / (nn3[d] - 1);
    }
    w.nn = (int64_t)ni * nj * nk;
    w.partial_slots = 16384;
#define TRY(x)                      \
    if ((rc = (x)) != ESPIC_OK) {   \
        free_world(w);              \
        delete h;                   \
        return rc;                  \
    }
    if (cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(ESPIC_ERR_CUDA, "cudaStreamCreate failed");
    }
    TRY(dalloc(&w.phi, w.nn));
    TRY(dalloc(&w.rho, w.nn));
    TRY(dalloc(&w.vol, w.nn));
    TRY(dalloc(&w.ivol, w.nn));
    TRY(dalloc(&w.ef, 3 * w.nn));
    TRY(dalloc(&w.ef4, w.nn));
    TRY(dalloc(&w.obj, w.nn));
    TRY(dalloc(&w.target, w.nn));
    TRY(dalloc(&w.d_err, 1));
    TRY(dalloc(&w.d_status, 1));
    TRY(dalloc(&w.d_partials, w.partial_slots));
    TRY(dalloc(&w.d_small, 256));
#undef TRY
    if (cudaMallocHost(&w.h_small, 256 * sizeof(double)) != cudaSuccess) {
        free_world(w);
        delete h;
        return fail(ESPIC_ERR_CUDA, "cudaMallocHost failed");
    }
    cudaMemsetAsync(w.phi, 0, w.nn * sizeof(double), w.stream);
    cudaMemsetAsync(w.rho, 0, w.nn * sizeof(double), w.stream);
    cudaMemsetAsync(w.ef, 0, 3 * w.nn * sizeof(double), w.stream);
    cudaMemsetAsync(w.ef4, 0, w.nn * sizeof(float4), w.stream);
    cudaMemsetAsync(w.obj, 0, w.nn * sizeof(int32_t), w.stream);
    cudaMemsetAsync(w.d_err, 0, sizeof(int), w.stream);
    cudaMemsetAsync(w.d_status, 0, sizeof(SolveStatus), w.stream);
    launch_node_vol(w);
    w.ef4_valid = true;
    if (cudaStreamSynchronize(w.stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        free_world(w);
        delete h;
        return fail(ESPIC_ERR_CUDA, "world initialisation failed");
    }
    *out = h;
    return ESPIC_OK;
}

extern "C" int espic_world_destroy(espic_world *h) {
    if (!h) return ESPIC_OK;
    cudaSetDevice(h->w.device);
    cudaStreamSynchronize(h->w.stream);
    free_world(h->w);
    delete h;
    return ESPIC_OK;
}

extern "C" int espic_world_set_time(espic_world *h, double dt, int num_ts) {
    WORLD(h);
    w.dt = dt;
    w.num_ts = num_ts;
    return ESPIC_OK;
}

extern "C" int espic_world_advance_time(espic_world *h) {
    WORLD(h);
    w.time += w.dt;
    w.ts++;
    return w.ts <= w.num_ts ? 1 : 0;
}

extern "C" int espic_world_get_time(espic_world *h, int *ts, double *time) {
    WORLD(h);
    if (ts) *ts = w.ts;
    if (time) *time = w.time;
    return ESPIC_OK;
}

extern "C" int espic_world_add_sphere(espic_world *h, const double c[3], double radius, double phi_sphere) {
    WORLD(h);
    if (!c || !(radius > 0)) return fail(ESPIC_ERR_ARG, "bad sphere");
    w.sphere[0] = c[0];
    w.sphere[1] = c[1];
    w.sphere[2] = c[2];
    w.sphere[3] = radius * radius;
    w.has_sphere = true;
    launch_objects_sphere(w, c, radius, phi_sphere);
    CHECK_LAUNCH();
    w.targets_valid = false;
    w.pcg_codes_valid = false;
    w.phi_prev_valid = false;
    return ESPIC_OK;
}

extern "C" int espic_world_add_inlet(espic_world *h) {
    WORLD(h);
    launch_objects_inlet(w);
    CHECK_LAUNCH();
    w.targets_valid = false;
    w.pcg_codes_valid = false;
    w.phi_prev_valid = false;
    return ESPIC_OK;
}

extern "C" int espic_world_set_seed(espic_world *h, uint64_t seed) {
    WORLD(h);
    w.seed = seed;
    return ESPIC_OK;
}

extern "C" int espic_world_sync(espic_world *h) {
    WORLD(h);
    CK(cudaStreamSynchronize(w.stream));
    CHECK_LAUNCH();
    return take_device_errors(w);
}

extern "C" int espic_world_stream(espic_world *h, void **stream) {
    WORLD(h);
    if (!stream) return fail(ESPIC_ERR_ARG, "null stream");
    *stream = (void *)w.stream;
    return ESPIC_OK;
}

/* ---------------------------------------------------------------- species */
static int fixed_exponent(double weight_bound, int64_t capacity) {
    if (capacity < 1) capacity = 1;
    if (!(weight_bound > 0)) weight_bound = 1;
    double lim = ldexp(1.0, 62) / ((double)capacity * weight_bound);
    int e;
    frexp(lim, &e);
    int S = e - 1;
    return S > 52 ? 52 : S;
}

static void set_weight_bound(Species &s, double wb) {
    s.weight_bound = wb;
    if (s.form == ESPIC_FORM_FP64) {
        s.fx = ldexp(1.0, fixed_exponent(wb, s.cap));
        s.unit = 1.0 / s.fx;
    }
}

extern "C" int espic_species_create(espic_world *h, double mass, double charge, double mpw0, int64_t capacity,
                                    int form, int walls, double weight_bound, int *species_id) {
    WORLD(h);
    if (!species_id) return fail(ESPIC_ERR_ARG, "null species_id");
    if (!(mass > 0)) return fail(ESPIC_ERR_ARG, "mass must be positive");
    if (capacity < 1 || capacity > 0x7fffffffLL) return fail(ESPIC_ERR_ARG, "capacity must be in [1, 2^31)");
    if (form != ESPIC_FORM_FP64 && form != ESPIC_FORM_MIXED) return fail(ESPIC_ERR_ARG, "unknown form");
    if (walls != ESPIC_WALLS_REFLECT && walls != ESPIC_WALLS_ABSORB) return fail(ESPIC_ERR_ARG, "unknown walls");
    if (form == ESPIC_FORM_MIXED) {
        if (!(mpw0 > 0)) return fail(ESPIC_ERR_ARG, "the mixed form needs a species weight mpw0 > 0");
        if (w.g.ni - 1 > 1024 || w.g.nj - 1 > 1024 || w.g.nk - 1 > 2047)
            return fail(ESPIC_ERR_ARG, "the mixed form's cell key holds at most 1024 x 1024 x 2047 cells");
    }
    if (w.species.size() >= 8) return fail(ESPIC_ERR_ARG, "at most 8 species");
    Species *s = new Species();
    s->id = (int)w.species.size();
    s->form = form;
    s->walls = walls;
    s->mass = mass;
    s->charge = charge;
    s->mpw0 = mpw0;
    s->cap = capacity;
    s->ms = (capacity + 63) / 64 * 64;
    int64_t words = capacity / 32 + 2;
    s->ntiles = capacity / TILE_PARTICLES + 2;
    int rc = ESPIC_OK;
#define TRY(x)                  \
    if ((rc = (x)) != ESPIC_OK) { \
        free_species(s);        \
        return rc;              \
    }
    if (form == ESPIC_FORM_FP64) {
        TRY(dalloc(&s->P, 7 * (size_t)capacity));
    } else {
        const int64_t ntiles =
            (int64_t)tile_count(w.g.ni - 1) * tile_count(w.g.nj - 1) * tile_count(w.g.nk - 1);
        const int64_t ncells = ntiles * TILE_CELLS * TILE_CELLS * TILE_CELLS; /* tile-major sort slots */
        TRY(dalloc(&s->seg, ntiles + 1));
        TRY(dalloc(&s->cell, s->ms));
        TRY(dalloc(&s->cell2, s->ms));
        TRY(dalloc(&s->off, 3 * (size_t)s->ms));
        TRY(dalloc(&s->off2, 3 * (size_t)s->ms));
        TRY(dalloc(&s->vel, 3 * (size_t)s->ms));
        TRY(dalloc(&s->vel2, 3 * (size_t)s->ms));
        TRY(dalloc(&s->sort_count, ncells + 2 + ncells / 8192 + 2));
    }
    TRY(dalloc(&s->deadmask, words));
    TRY(dalloc(&s->tiledead, s->ntiles + 1));
    TRY(dalloc(&s->tilepre, s->ntiles + 1));
    TRY(dalloc(&s->holes, capacity));
    TRY(dalloc(&s->d_count, 4));
    TRY(dalloc(&s->acc, w.nn));
    TRY(dalloc(&s->den, w.nn));
    TRY(dalloc(&s->den_ave, w.nn));
#undef TRY
    cudaMemsetAsync(s->tiledead, 0, (s->ntiles + 1) * sizeof(int32_t), w.stream);
    cudaMemsetAsync(s->d_count, 0, 4 * sizeof(int64_t), w.stream);
    cudaMemsetAsync(s->acc, 0, w.nn * sizeof(unsigned long long), w.stream);
    cudaMemsetAsync(s->den, 0, w.nn * sizeof(double), w.stream);
    cudaMemsetAsync(s->den_ave, 0, w.nn * sizeof(double), w.stream);
    if (form == ESPIC_FORM_MIXED) {
        s->unit = mpw0 / 8388608.0; /* counts of mpw0 * 2^-23 */
        s->weight_bound = mpw0;
        if (!w.ef4_valid) launch_ef4(w);
    } else {
        double wb = weight_bound > 0 ? weight_bound : mpw0;
        if (wb > 0) set_weight_bound(*s, wb);
    }
    s->uniform_w = mpw0 > 0;
    CHECK_LAUNCH();
    w.species.push_back(s);
    *species_id = s->id;
    return ESPIC_OK;
}

extern "C" int espic_species_count(espic_world *h, int sp, int64_t *np) {
    WORLD(h);
    SPECIES(sp);
    if (!np) return fail(ESPIC_ERR_ARG, "null np");
    int64_t n = 0;
    CK(cudaMemcpyAsync(&n, s.d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    s.host_bound = n;
    *np = n;
    return take_device_errors(w);
}

static int ensure_stage(World &w, int64_t doubles) {
    if (w.d_stage_cap >= doubles) return ESPIC_OK;
    if (w.d_stage) {
        cudaStreamSynchronize(w.stream);
        cudaFree(w.d_stage);
    }
    w.d_stage = nullptr;
    w.d_stage_cap = 0;
    int rc = dalloc(&w.d_stage, (size_t)doubles);
    if (rc == ESPIC_OK) w.d_stage_cap = doubles;
    return rc;
}

static int ensure_u(World &w, int64_t doubles) {
    if (w.d_u_cap >= doubles) return ESPIC_OK;
    if (w.d_u) {
        cudaStreamSynchronize(w.stream);
        cudaFree(w.d_u);
    }
    w.d_u = nullptr;
    w.d_u_cap = 0;
    int rc = dalloc(&w.d_u, (size_t)doubles);
    if (rc == ESPIC_OK) w.d_u_cap = doubles;
    return rc;
}

/* a float64 species that receives weights other than mpw0 keeps a weight row */
static int make_nonuniform(World &w, Species &s) {
    if (!s.uniform_w) return ESPIC_OK;
    if (s.form != ESPIC_FORM_FP64) return fail(ESPIC_ERR_ARG, "the mixed form holds one weight per species");
    launch_fill(w, s.P + 6 * s.cap, s.cap, s.mpw0);
    s.uniform_w = false;
    CHECK_LAUNCH();
    return ESPIC_OK;
}

static int prepare_weights(World &w, Species &s, const double *wts, int64_t n, double single) {
    double wmax = single;
    bool differs = wts == nullptr ? (single != s.mpw0) : false;
    if (wts) {
        wmax = 0;
        for (int64_t i = 0; i < n; i++) {
            wmax = std::max(wmax, fabs(wts[i]));
            if (wts[i] != s.mpw0) differs = true;
        }
    }
    if (!(s.weight_bound > 0)) set_weight_bound(s, wmax > 0 ? wmax : 1.0);
    if (s.form == ESPIC_FORM_FP64 && wmax * s.fx > ldexp(1.0, 62) / (double)s.cap)
        return fail(ESPIC_ERR_FIXED, "weight %g exceeds the fixed-point bound of this species", wmax);
    if (differs) return make_nonuniform(w, s);
    return ESPIC_OK;
}

extern "C" int espic_species_add(espic_world *h, int sp, const double *pos3, const double *vel3,
                                 const double *mpw, int64_t n) {
    WORLD(h);
    SPECIES(sp);
    if (n < 0 || (n > 0 && (!pos3 || !vel3))) return fail(ESPIC_ERR_ARG, "bad particle arrays");
    if (n == 0) return ESPIC_OK;
    int rc = prepare_weights(w, s, mpw, n, s.mpw0);
    if (rc != ESPIC_OK) return rc;
    if ((rc = ensure_stage(w, 7 * n)) != ESPIC_OK) return rc;
    double *dp = w.d_stage, *dv = w.d_stage + 3 * n, *dw = mpw ? w.d_stage + 6 * n : nullptr;
    CK(cudaMemcpyAsync(dp, pos3, 3 * n * sizeof(double), cudaMemcpyHostToDevice, w.stream));
    CK(cudaMemcpyAsync(dv, vel3, 3 * n * sizeof(double), cudaMemcpyHostToDevice, w.stream));
    if (mpw) CK(cudaMemcpyAsync(dw, mpw, n * sizeof(double), cudaMemcpyHostToDevice, w.stream));
    launch_add_fp64(w, s, dp, dv, dw, n, 1);
    CHECK_LAUNCH();
    CK(cudaStreamSynchronize(w.stream)); /* the host arrays may be reused on return */
    return take_device_errors(w);
}

extern "C" int espic_species_set(espic_world *h, int sp, const double *P, int64_t stride, int64_t n) {
    WORLD(h);
    SPECIES(sp);
    if (n < 0 || n > s.cap) return fail(ESPIC_ERR_CAPACITY, "%lld particles exceed the capacity", (long long)n);
    if (n > 0 && (!P || stride < n)) return fail(ESPIC_ERR_ARG, "bad particle block");
    int rc;
    if (n > 0) {
        rc = prepare_weights(w, s, P + 6 * stride, n, s.mpw0);
        if (rc != ESPIC_OK) return rc;
    }
    if (s.form == ESPIC_FORM_FP64) {
        int rows = s.uniform_w ? 6 : 7;
        if (n > 0)
            CK(cudaMemcpy2DAsync(s.P, s.cap * sizeof(double), P, stride * sizeof(double), n * sizeof(double), rows,
                                 cudaMemcpyHostToDevice, w.stream));
    } else if (n > 0) {
        if ((rc = ensure_stage(w, 7 * n)) != ESPIC_OK) return rc;
        CK(cudaMemcpy2DAsync(w.d_stage, n * sizeof(double), P, stride * sizeof(double), n * sizeof(double), 6,
                             cudaMemcpyHostToDevice, w.stream));
        launch_to_mixed(w, s, w.d_stage, n, 0, n);
        CHECK_LAUNCH();
    }
    int64_t cnt[4] = {n, n, 0, 0};
    CK(cudaMemcpyAsync(s.d_count, cnt, sizeof cnt, cudaMemcpyHostToDevice, w.stream));
    s.tiled = false; /* new particle order: no tile segments until the next sort */
    s.dsum_valid = false;
    /* for the ch4 push, particles set here have a step's time left */
    if (s.ch4_settled) CK(cudaMemsetAsync(s.ch4_settled, 0, sizeof(int64_t), w.stream));
    CK(cudaStreamSynchronize(w.stream));
    s.host_bound = n;
    return take_device_errors(w);
}

extern "C" int espic_species_get(espic_world *h, int sp, double *P, int64_t stride, int64_t cap, int64_t *np) {
    WORLD(h);
    SPECIES(sp);
    int64_t n = 0;
    CK(cudaMemcpyAsync(&n, s.d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    s.host_bound = n;
    if (np) *np = n;
    if (!P) return take_device_errors(w);
    if (n > cap || stride < n) return fail(ESPIC_ERR_CAPACITY, "output holds %lld of %lld particles", (long long)cap,
                                         (long long)n);
    if (n > 0) {
        if (s.form == ESPIC_FORM_FP64) {
            int rows = s.uniform_w ? 6 : 7;
            CK(cudaMemcpy2DAsync(P, stride * sizeof(double), s.P, s.cap * sizeof(double), n * sizeof(double), rows,
                                 cudaMemcpyDeviceToHost, w.stream));
            CK(cudaStreamSynchronize(w.stream));
            if (s.uniform_w)
                for (int64_t i = 0; i < n; i++) P[6 * stride + i] = s.mpw0;
        } else {
            int rc = ensure_stage(w, 7 * n);
            if (rc != ESPIC_OK) return rc;
            launch_from_mixed(w, s, w.d_stage, n, n);
            CHECK_LAUNCH();
            CK(cudaMemcpy2DAsync(P, stride * sizeof(double), w.d_stage, n * sizeof(double), n * sizeof(double), 7,
                                 cudaMemcpyDeviceToHost, w.stream));
            CK(cudaStreamSynchronize(w.stream));
        }
    }
    return take_device_errors(w);
}

extern "C" int espic_species_set_mixed(espic_world *h, int sp, const int32_t *cell, const float *off,
                                       const float *vel, int64_t stride, int64_t n) {
    WORLD(h);
    SPECIES(sp);
    if (s.form != ESPIC_FORM_MIXED) return fail(ESPIC_ERR_ARG, "the species is not in the mixed form");
    if (n < 0 || n > s.cap) return fail(ESPIC_ERR_CAPACITY, "%lld particles exceed the capacity", (long long)n);
    if (n > 0 && (!cell || !off || !vel || stride < n)) return fail(ESPIC_ERR_ARG, "bad mixed particle block");
    /* every key must name a cell and every offset lie in [0,1] (1 itself
     * occurs when an offset just below 1 rounds up to float): the kernels
     * index the node fields with them */
    for (int64_t p = 0; p < n; p++) {
        const int32_t key = cell[p];
        const int i = key & 1023, j = (key >> 10) & 1023, k = key >> 20;
        if (key < 0 || i > w.g.ni - 2 || j > w.g.nj - 2 || k > w.g.nk - 2)
            return fail(ESPIC_ERR_ARG, "particle %lld: cell key %d names no cell of the grid", (long long)p, key);
        for (int d = 0; d < 3; d++) {
            const float f = off[d * stride + p];
            if (!(f >= 0.f && f <= 1.f))
                return fail(ESPIC_ERR_ARG, "particle %lld: in-cell offset outside [0,1]", (long long)p);
        }
    }
    s.dsum_valid = false;
    if (n > 0) {
        CK(cudaMemcpyAsync(s.cell, cell, n * sizeof(int32_t), cudaMemcpyHostToDevice, w.stream));
        CK(cudaMemcpy2DAsync(s.off, s.ms * sizeof(float), off, stride * sizeof(float), n * sizeof(float), 3,
                             cudaMemcpyHostToDevice, w.stream));
        CK(cudaMemcpy2DAsync(s.vel, s.ms * sizeof(float), vel, stride * sizeof(float), n * sizeof(float), 3,
                             cudaMemcpyHostToDevice, w.stream));
    }
    int64_t cnt[4] = {n, n, 0, 0};
    CK(cudaMemcpyAsync(s.d_count, cnt, sizeof cnt, cudaMemcpyHostToDevice, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    s.host_bound = n;
    s.tiled = false;
    return take_device_errors(w);
}

extern "C" int espic_species_get_mixed(espic_world *h, int sp, int32_t *cell, float *off, float *vel, int64_t stride,
                                       int64_t cap, int64_t *np) {
    WORLD(h);
    SPECIES(sp);
    if (s.form != ESPIC_FORM_MIXED) return fail(ESPIC_ERR_ARG, "the species is not in the mixed form");
    int64_t n = 0;
    CK(cudaMemcpyAsync(&n, s.d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    s.host_bound = n;
    if (np) *np = n;
    if (!cell) return take_device_errors(w);
    if (!off || !vel) return fail(ESPIC_ERR_ARG, "null offset or velocity block");
    if (n > cap || stride < n) return fail(ESPIC_ERR_CAPACITY, "output holds %lld of %lld particles", (long long)cap,
                                         (long long)n);
    if (n > 0) {
        CK(cudaMemcpyAsync(cell, s.cell, n * sizeof(int32_t), cudaMemcpyDeviceToHost, w.stream));
        CK(cudaMemcpy2DAsync(off, stride * sizeof(float), s.off, s.ms * sizeof(float), n * sizeof(float), 3,
                             cudaMemcpyDeviceToHost, w.stream));
        CK(cudaMemcpy2DAsync(vel, stride * sizeof(float), s.vel, s.ms * sizeof(float), n * sizeof(float), 3,
                             cudaMemcpyDeviceToHost, w.stream));
        CK(cudaStreamSynchronize(w.stream));
    }
    return take_device_errors(w);
}

extern "C" int espic_species_load_box(espic_world *h, int sp, const double x1[3], const double x2[3],
                                      double num_den, int64_t num_mp, const double *u) {
    WORLD(h);
    SPECIES(sp);
    if (!x1 || !x2 || num_mp < 0) return fail(ESPIC_ERR_ARG, "bad load box");
    if (num_mp == 0) return ESPIC_OK;
    double box_vol = (x2[0] - x1[0]) * (x2[1] - x1[1]) * (x2[2] - x1[2]);
    double num_real = num_den * box_vol;
    double mpw = num_real / (double)num_mp;
    int rc = prepare_weights(w, s, nullptr, 1, mpw);
    if (rc != ESPIC_OK) return rc;
    const double *du = nullptr;
    if (u) {
        if ((rc = ensure_u(w, 3 * num_mp)) != ESPIC_OK) return rc;
        CK(cudaMemcpyAsync(w.d_u, u, 3 * num_mp * sizeof(double), cudaMemcpyHostToDevice, w.stream));
        du = w.d_u;
    }
    uint64_t stream_id = ((uint64_t)(0x10000u + w.load_calls++) << 32);
    launch_load_box(w, s, x1, x2, mpw, num_mp, du, stream_id);
    CHECK_LAUNCH();
    CK(cudaStreamSynchronize(w.stream));
    return take_device_errors(w);
}

extern "C" int espic_species_load_box_thermal(espic_world *h, int sp, const double x1[3], const double x2[3],
                                              double mpw, int64_t num_mp, const double v_drift[3], double temp,
                                              const double *u) {
    WORLD(h);
    SPECIES(sp);
    if (!x1 || !x2 || !v_drift || num_mp < 0 || temp < 0 || mpw < 0) return fail(ESPIC_ERR_ARG, "bad thermal load");
    if (num_mp == 0) return ESPIC_OK;
    if (mpw == 0) mpw = s.mpw0;
    if (!(mpw > 0)) return fail(ESPIC_ERR_ARG, "no weight: give mpw or a species mpw0");
    int rc = prepare_weights(w, s, nullptr, 1, mpw);
    if (rc != ESPIC_OK) return rc;
    const double *du = nullptr;
    if (u) {
        if ((rc = ensure_u(w, 7 * num_mp)) != ESPIC_OK) return rc;
        CK(cudaMemcpyAsync(w.d_u, u, 7 * num_mp * sizeof(double), cudaMemcpyHostToDevice, w.stream));
        du = w.d_u;
    }
    uint64_t stream_id = ((uint64_t)(0x20000u + w.load_calls++) << 32);
    PhaseScope ph(w, ESPIC_PHASE_INJECT);
    launch_load_thermal(w, s, x1, x2, mpw, num_mp, v_drift, temp, du, stream_id);
    CHECK_LAUNCH();
    CK(cudaStreamSynchronize(w.stream));
    return take_device_errors(w);
}

extern "C" int espic_species_load_box_qs(espic_world *h, int sp, const double x1[3], const double x2[3],
                                         double num_den, const int num_mp[3]) {
    WORLD(h);
    SPECIES(sp);
    if (!x1 || !x2 || !num_mp || num_mp[0] < 2 || num_mp[1] < 2 || num_mp[2] < 2)
        return fail(ESPIC_ERR_ARG, "bad quiet-start load");
    double box_vol = (x2[0] - x1[0]) * (x2[1] - x1[1]) * (x2[2] - x1[2]);
    int num_mp_tot = (num_mp[0] - 1) * (num_mp[1] - 1) * (num_mp[2] - 1);
    double num_real = num_den * box_vol;
    double mpw = num_real / num_mp_tot;
    /* edge particles carry mpw/2..mpw/8: per-particle weights */
    int rc = prepare_weights(w, s, nullptr, 1, mpw);
    if (rc != ESPIC_OK) return rc;
    if ((rc = make_nonuniform(w, s)) != ESPIC_OK) return rc;
    launch_load_qs(w, s, x1, x2, mpw, num_mp);
    CHECK_LAUNCH();
    CK(cudaStreamSynchronize(w.stream));
    return take_device_errors(w);
}

/* ---------------------------------------------------------------- the step */
static void ensure_ef4(World &w) {
    if (!w.ef4_valid) launch_ef4(w);
}

static int push_one(World &w, Species &s, bool deposit) {
    if (deposit) {
        PhaseScope ph(w, ESPIC_PHASE_DENSITY);
        CK(cudaMemsetAsync(s.acc, 0, w.nn * sizeof(unsigned long long), w.stream));
    }
    if (s.form != ESPIC_FORM_FP64) ensure_ef4(w);
    {
        PhaseScope ph(w, ESPIC_PHASE_PUSH);
        if (s.form == ESPIC_FORM_FP64)
            launch_push_fp64(w, s, deposit);
        else
            launch_push_mixed(w, s, deposit);
    }
    CHECK_LAUNCH();
    if (s.walls == ESPIC_WALLS_ABSORB) {
        PhaseScope ph(w, ESPIC_PHASE_COMPACT);
        launch_compact(w, s);
        CHECK_LAUNCH();
    }
    if (deposit) {
        PhaseScope ph(w, ESPIC_PHASE_DENSITY);
        launch_density(w, s);
        CHECK_LAUNCH();
    }
    return ESPIC_OK;
}

extern "C" int espic_push(espic_world *h, int sp, int deposit) {
    WORLD(h);
    SPECIES(sp);
    if (deposit && !(s.weight_bound > 0)) set_weight_bound(s, 1.0);
    return push_one(w, s, deposit != 0);
}

extern "C" int espic_deposit(espic_world *h, int sp) {
    WORLD(h);
    SPECIES(sp);
    if (!(s.weight_bound > 0)) set_weight_bound(s, 1.0);
    CK(cudaMemsetAsync(s.acc, 0, w.nn * sizeof(unsigned long long), w.stream));
    if (s.form == ESPIC_FORM_FP64)
        launch_deposit_fp64(w, s);
    else
        launch_deposit_mixed(w, s);
    CHECK_LAUNCH();
    launch_density(w, s);
    CHECK_LAUNCH();
    return ESPIC_OK;
}

extern "C" int espic_charge_density(espic_world *h) {
    WORLD(h);
    PhaseScope ph(w, ESPIC_PHASE_DENSITY);
    launch_charge(w);
    w.rho_version++;
    CHECK_LAUNCH();
    return ESPIC_OK;
}

extern "C" int espic_sort(espic_world *h, int sp) {
    WORLD(h);
    SPECIES(sp);
    if (s.form != ESPIC_FORM_MIXED) return ESPIC_OK;
    PhaseScope ph(w, ESPIC_PHASE_SORT);
    launch_sort_mixed(w, s);
    CHECK_LAUNCH();
    return ESPIC_OK;
}

extern "C" int espic_source_create(espic_world *h, int sp, double v_drift, double den, double temp,
                                   int *source_id) {
    WORLD(h);
    SPECIES(sp);
    if (!source_id) return fail(ESPIC_ERR_ARG, "null source_id");
    if (!(s.mpw0 > 0)) return fail(ESPIC_ERR_ARG, "a source needs a species weight mpw0 > 0");
    if (temp < 0) return fail(ESPIC_ERR_ARG, "negative temperature");
    Source src;
    src.sp = sp;
    src.v_drift = v_drift;
    src.den = den;
    src.temp = temp;
    src.vmode = temp > 0 ? ESPIC_BEAM_WARM : ESPIC_BEAM_COLD;
    src.count_mode = ESPIC_COUNT_RANDOM;
    w.sources.push_back(src);
    *source_id = (int)w.sources.size() - 1;
    return ESPIC_OK;
}

/* ColdBeamSource::sample, ch3/ver2/Source.cpp:7-18: (int)(n v A dt/mpw0 + U) */
/* macroparticles of one sample: (int)(N_real / mpw0 + U) (ch3/ver2/Source.cpp:
 * 18) or, with the remainder count, (int)(N_real / mpw0 + remainder) with the
 * fraction carried to the next call (ch9/MPI/src/Source.cpp:20-27) */
static int inject_count(const World &w, Source &src, double mpw0, double u0) {
    if (src.count_mode == ESPIC_COUNT_REMAINDER) {
        /* ch9/MPI/src/Source.cpp:10-27, in its own operand order */
        const double area = (w.g.ni - 1) * w.g.dh[0] * (w.g.nj - 1) * w.g.dh[1];
        const double num_per_sec = src.den * src.v_drift * area;
        const double num_real = num_per_sec * w.dt;
        double f = num_real / mpw0 + src.remainder;
        int n = (int)f;
        src.remainder = f - n;
        return n;
    }
    double Lx = w.g.dh[0] * (w.g.ni - 1);
    double Ly = w.g.dh[1] * (w.g.nj - 1);
    double A = Lx * Ly;
    double num_real = src.den * src.v_drift * A * w.dt;
    return (int)(num_real / mpw0 + u0);
}

extern "C" int espic_source_sample(espic_world *h, int source) {
    WORLD(h);
    if (source < 0 || source >= (int)w.sources.size()) return fail(ESPIC_ERR_ARG, "bad source id");
    Source &src = w.sources[source];
    Species &s = *w.species[src.sp];
    uint64_t stream_id = ((uint64_t)(source + 1) << 32) | (uint32_t)src.calls;
    src.calls++;
    double u0 = philox_uniform(w.seed, stream_id, 0);
    int num_sim = inject_count(w, src, s.mpw0, u0);
    if (num_sim <= 0) return ESPIC_OK;
    PhaseScope ph(w, ESPIC_PHASE_INJECT);
    launch_inject(w, s, num_sim, src.v_drift, src.temp, src.vmode, nullptr, stream_id);
    CHECK_LAUNCH();
    return ESPIC_OK;
}

extern "C" int espic_source_sample_uniforms(espic_world *h, int source, const double *u, int64_t nu,
                                            int64_t *used) {
    WORLD(h);
    if (source < 0 || source >= (int)w.sources.size()) return fail(ESPIC_ERR_ARG, "bad source id");
    if (!u || nu < 1) return fail(ESPIC_ERR_ARG, "need at least the count uniform");
    Source &src = w.sources[source];
    Species &s = *w.species[src.sp];
    int num_sim = inject_count(w, src, s.mpw0, u[0]);
    int64_t upp = beam_uniforms(src.vmode);
    int64_t need = 1 + upp * (int64_t)(num_sim > 0 ? num_sim : 0);
    if (nu < need) return fail(ESPIC_ERR_ARG, "%lld uniforms given, %lld needed", (long long)nu, (long long)need);
    if (used) *used = need;
    if (num_sim <= 0) return ESPIC_OK;
    int rc = ensure_u(w, need);
    if (rc != ESPIC_OK) return rc;
    CK(cudaMemcpyAsync(w.d_u, u, need * sizeof(double), cudaMemcpyHostToDevice, w.stream));
    PhaseScope ph(w, ESPIC_PHASE_INJECT);
    launch_inject(w, s, num_sim, src.v_drift, src.temp, src.vmode, w.d_u, 0);
    CHECK_LAUNCH();
    CK(cudaStreamSynchronize(w.stream));
    return take_device_errors(w);
}

extern "C" int espic_source_set_mode(espic_world *h, int source, int velocity_mode, int count_mode) {
    WORLD(h);
    if (source < 0 || source >= (int)w.sources.size()) return fail(ESPIC_ERR_ARG, "bad source id");
    if (velocity_mode < ESPIC_BEAM_COLD || velocity_mode > ESPIC_BEAM_MAXWELLIAN)
        return fail(ESPIC_ERR_ARG, "unknown velocity mode");
    if (count_mode != ESPIC_COUNT_RANDOM && count_mode != ESPIC_COUNT_REMAINDER)
        return fail(ESPIC_ERR_ARG, "unknown count mode");
    Source &src = w.sources[source];
    if (velocity_mode != ESPIC_BEAM_COLD && !(src.temp > 0))
        return fail(ESPIC_ERR_ARG, "a thermal velocity mode needs a temperature > 0");
    src.vmode = velocity_mode;
    src.count_mode = count_mode;
    src.remainder = 0;
    return ESPIC_OK;
}

/* ---------------------------------------------------------------- solver */
extern "C" int espic_solver_set(espic_world *h, int kind, int max_it, double tol) {
    WORLD(h);
    if (kind < ESPIC_SOLVER_SOR || kind > ESPIC_SOLVER_QN) return fail(ESPIC_ERR_ARG, "unknown solver");
    if (max_it < 0 || !(tol >= 0)) return fail(ESPIC_ERR_ARG, "bad max_it / tol");
    w.solver_kind = kind;
    w.max_it = max_it;
    w.tol = tol;
    return ESPIC_OK;
}

extern "C" int espic_solver_set_reference(espic_world *h, double phi0, double te0, double n0) {
    WORLD(h);
    if (!(te0 > 0)) return fail(ESPIC_ERR_ARG, "Te0 must be positive");
    w.phi0 = phi0;
    w.te0 = te0;
    w.n0 = n0;
    return ESPIC_OK;
}

extern "C" int espic_solver_set_newton(espic_world *h, int nr_max, double nr_tol, int pcg_max, double pcg_tol,
                                       int fp32_inner) {
    WORLD(h);
    if (nr_max < 1 || pcg_max < 1 || !(nr_tol >= 0) || !(pcg_tol >= 0)) return fail(ESPIC_ERR_ARG, "bad Newton controls");
    w.nr_max = nr_max;
    w.nr_tol = nr_tol;
    w.pcg_max = pcg_max;
    w.pcg_tol = pcg_tol;
    w.fp32_inner = fp32_inner != 0;
    return ESPIC_OK;
}

extern "C" int espic_solver_set_multigrid(espic_world *h, int levels, double scale) {
    WORLD(h);
    if (levels < 0 || levels > 12 || !(scale > 0 && scale < 2)) return fail(ESPIC_ERR_ARG, "bad multigrid controls");
    if (levels != w.mg_levels_max) w.pcg_codes_valid = false; /* levels to set up change */
    w.mg_levels_max = levels;
    w.mg_scale = scale;
    return ESPIC_OK;
}

extern "C" int espic_solver_set_fallback(espic_world *h, int enable) {
    WORLD(h);
    w.gs_fallback = enable != 0;
    return ESPIC_OK;
}

extern "C" int espic_solver_status(espic_world *h, int *converged, int *iterations, int *inner_iterations,
                                   int *fallback_sweeps, double *residual) {
    WORLD(h);
    SolveStatus st;
    CK(cudaMemcpyAsync(&st, w.d_status, sizeof st, cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    if (converged) *converged = st.converged;
    if (iterations) *iterations = st.iterations;
    if (inner_iterations) *inner_iterations = st.inner_iterations;
    if (fallback_sweeps) *fallback_sweeps = st.fallback_sweeps;
    if (residual) *residual = st.residual;
    return take_device_errors(w);
}

extern "C" int espic_solver_set_coarse(espic_world *h, int64_t block_nodes) {
    WORLD(h);
    if (block_nodes < 0) return fail(ESPIC_ERR_ARG, "bad coarse-level size");
    w.mg_block_nodes = block_nodes;
    return ESPIC_OK;
}

extern "C" int espic_solver_set_dense(espic_world *h, int64_t max_nodes) {
    WORLD(h);
    if (max_nodes < 0 || max_nodes > 4096) return fail(ESPIC_ERR_ARG, "bad dense coarse-level size");
    if (max_nodes != w.mg_dense_max) {
        w.mg_dense_max = max_nodes;
        w.pcg_codes_valid = false; /* the hierarchy and its setup change */
    }
    return ESPIC_OK;
}

extern "C" int espic_solver_set_predictor(espic_world *h, int enable) {
    WORLD(h);
    w.predictor = enable != 0;
    w.phi_prev_valid = false;
    return ESPIC_OK;
}

extern "C" int espic_solver_set_launch(espic_world *h, int max_blocks) {
    WORLD(h);
    if (max_blocks < 0) return fail(ESPIC_ERR_ARG, "bad block count");
    w.solver_blocks = max_blocks;
    return ESPIC_OK;
}

static int enqueue_solve(World &w) {
    PhaseScope ph(w, ESPIC_PHASE_SOLVE);
    int e = 0;
    switch (w.solver_kind) {
        case ESPIC_SOLVER_SOR:
            e = launch_sor_box(w, w.max_it, w.tol);
            break;
        case ESPIC_SOLVER_GS:
        case ESPIC_SOLVER_PCG:
            if (!w.targets_valid) {
                launch_targets(w);
                w.targets_valid = true;
            }
            if (w.solver_kind == ESPIC_SOLVER_PCG && w.predictor) {
                /* predictor: between consecutive steps (one new charge
                 * density since the last solve) the Newton solve starts
                 * from 2 phi^n - phi^(n-1); otherwise from phi^n */
                /* two rows: the float-inner solve's quadratic predictor keeps
                 * the last two potentials */
                if (!w.phi_prev && cudaMalloc(&w.phi_prev, 2 * w.nn * sizeof(double)) != cudaSuccess) {
                    w.phi_prev = nullptr;
                    w.predictor = false;
                }
                if (w.phi_prev) {
                    bool extrapolate = w.phi_prev_valid && w.rho_version == w.solve_rho_version + 1;
                    if (w.fp32_inner) { /* the float-inner solve does it in its first pass */
                        w.predict_mode = !extrapolate ? 1 : (w.phi_prev2_valid ? 3 : 2);
                        w.phi_prev2_valid = extrapolate;
                    } else {
                        launch_predict(w, extrapolate);
                        w.phi_prev2_valid = false;
                    }
                    w.phi_prev_valid = true;
                    w.solve_rho_version = w.rho_version;
                }
            }
            e = w.solver_kind == ESPIC_SOLVER_GS ? launch_gs_sphere(w, w.max_it, w.tol)
                                                 : launch_newton_pcg(w, w.fp32_inner != 0);
            w.predict_mode = 0;
            break;
        case ESPIC_SOLVER_QN: {
            launch_qn(w);
            SolveStatus st;
            CK(cudaMemcpyAsync(&st, w.d_status, sizeof st, cudaMemcpyDeviceToHost, w.stream));
            CK(cudaStreamSynchronize(w.stream));
            st.converged = 1;
            st.iterations = 1;
            st.inner_iterations = 0;
            st.residual = 0;
            st.solves += 1;
            st.outer_total += 1;
            CK(cudaMemcpyAsync(w.d_status, &st, sizeof st, cudaMemcpyHostToDevice, w.stream));
            CK(cudaStreamSynchronize(w.stream));
            break;
        }
    }
    if (e) return fail(ESPIC_ERR_CUDA, "solver launch: %s", cudaGetErrorString((cudaError_t)e));
    CHECK_LAUNCH();
    return ESPIC_OK;
}

extern "C" int espic_solve(espic_world *h, int *iterations, int *inner_iterations, double *residual) {
    WORLD(h);
    int rc = enqueue_solve(w);
    if (rc != ESPIC_OK) return rc;
    if (!iterations && !inner_iterations && !residual) return ESPIC_OK;
    SolveStatus st;
    CK(cudaMemcpyAsync(&st, w.d_status, sizeof st, cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    if ((rc = take_device_errors(w)) != ESPIC_OK) return rc;
    if (iterations) *iterations = st.iterations;
    if (inner_iterations) *inner_iterations = st.inner_iterations;
    if (residual) *residual = st.residual;
    return st.converged ? ESPIC_OK : ESPIC_NOT_CONVERGED;
}

extern "C" int espic_efield(espic_world *h) {
    WORLD(h);
    PhaseScope ph(w, ESPIC_PHASE_EFIELD);
    launch_efield(w, false);
    CHECK_LAUNCH();
    return ESPIC_OK;
}

/* ---------------------------------------------------------------- diagnostics */
/* ---------------------------------------------------------------- DSMC_MEX */
extern "C" int espic_dsmc_enable(espic_world *h, int sp, const double *c, double sigma_cr_max) {
    WORLD(h);
    SPECIES(sp);
    if (s.form != 0) return fail(ESPIC_ERR_ARG, "DSMC works on a species in the float64 form");
    if (!(sigma_cr_max > 0)) return fail(ESPIC_ERR_ARG, "sigma_cr_max must be positive");
    if (c) {
        for (int d = 0; d < 4; d++) s.dsmc_c[d] = c[d];
    } else {
        /* the reference's constructor, ch4/Collisions.h:53-60 (Bird's VHS
         * parameters at 273.15 K; m_r of a like pair) */
        const double K = 1.380648e-23;
        const double mr = s.mass * s.mass / (s.mass + s.mass);
        s.dsmc_c[0] = 4.07e-10;
        s.dsmc_c[1] = 0.77;
        s.dsmc_c[2] = 2 * K * 273.15 / mr;
        s.dsmc_c[3] = tgamma(2.5 - s.dsmc_c[1]);
    }
    const int64_t n_cells = (int64_t)(w.g.ni - 1) * (w.g.nj - 1) * (w.g.nk - 1);
    if (!s.dsmc_on) {
        if (dalloc(&s.d_dsmc, 4) != ESPIC_OK || dalloc(&s.dsmc_cell, s.cap) != ESPIC_OK ||
            dalloc(&s.dsmc_rank, s.cap) != ESPIC_OK || dalloc(&s.dsmc_perm, s.cap) != ESPIC_OK ||
            dalloc(&s.dsmc_count, n_cells + 1) != ESPIC_OK || dalloc(&s.dsmc_start, n_cells + 1) != ESPIC_OK ||
            dalloc(&s.dsmc_bsum, int_scan_blocks(n_cells) + 1) != ESPIC_OK)
            return ESPIC_ERR_CUDA;
        s.dsmc_on = true;
    }
    unsigned long long st[4] = {0, 0, 0, 0};
    memcpy(&st[0], &sigma_cr_max, sizeof(double));
    CK(cudaMemcpyAsync(s.d_dsmc, st, sizeof st, cudaMemcpyHostToDevice, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    return ESPIC_OK;
}

extern "C" int espic_dsmc_apply(espic_world *h, int sp, double dt, const double *u, int64_t nu,
                                const int64_t *cell_off) {
    WORLD(h);
    SPECIES(sp);
    if (!s.dsmc_on) return fail(ESPIC_ERR_ARG, "DSMC not enabled on species %d", sp);
    if (!(dt > 0)) return fail(ESPIC_ERR_ARG, "bad time step");
    if (!u) {
        launch_dsmc(w, s, dt, nullptr, 0, nullptr);
        CHECK_LAUNCH();
        return ESPIC_OK;
    }
    /* replayed uniforms (parity checks): staged for this call */
    if (!cell_off || nu < 0) return fail(ESPIC_ERR_ARG, "replayed uniforms need their cell offsets");
    const int64_t n_cells = (int64_t)(w.g.ni - 1) * (w.g.nj - 1) * (w.g.nk - 1);
    double *du = nullptr;
    int64_t *doff = nullptr;
    if (dalloc(&du, nu) != ESPIC_OK) return ESPIC_ERR_CUDA;
    if (dalloc(&doff, n_cells + 1) != ESPIC_OK) {
        cudaFree(du);
        return ESPIC_ERR_CUDA;
    }
    cudaMemcpyAsync(du, u, nu * sizeof(double), cudaMemcpyHostToDevice, w.stream);
    cudaMemcpyAsync(doff, cell_off, (n_cells + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, w.stream);
    launch_dsmc(w, s, dt, du, nu, doff);
    cudaError_t e = cudaStreamSynchronize(w.stream);
    cudaFree(du);
    cudaFree(doff);
    if (e != cudaSuccess) return fail(ESPIC_ERR_CUDA, "%s", cudaGetErrorString(e));
    CHECK_LAUNCH();
    return take_device_errors(w);
}

extern "C" int espic_dsmc_status(espic_world *h, int sp, double *sigma_cr_max, int64_t *collisions_last,
                                 int64_t *collisions_total) {
    WORLD(h);
    SPECIES(sp);
    if (!s.dsmc_on) return fail(ESPIC_ERR_ARG, "DSMC not enabled on species %d", sp);
    unsigned long long st[4];
    CK(cudaMemcpyAsync(st, s.d_dsmc, sizeof st, cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    if (sigma_cr_max) memcpy(sigma_cr_max, &st[0], sizeof(double));
    if (collisions_last) *collisions_last = (int64_t)st[2];
    if (collisions_total) *collisions_total = (int64_t)st[3];
    return take_device_errors(w);
}

/* ---------------------------------------------------------------- ch4 moments, MCC */
static int ensure_ch4(World &w, Species &s);

extern "C" int espic_sample_moments(espic_world *h, int sp) {
    WORLD(h);
    SPECIES(sp);
    int rc = ensure_ch4(w, s);
    if (rc != ESPIC_OK) return rc;
    launch_moments(w, s);
    CHECK_LAUNCH();
    return ESPIC_OK;
}

extern "C" int espic_gas_properties(espic_world *h, int sp) {
    WORLD(h);
    SPECIES(sp);
    int rc = ensure_ch4(w, s);
    if (rc != ESPIC_OK) return rc;
    launch_gas_props(w, s);
    CHECK_LAUNCH();
    return ESPIC_OK;
}

extern "C" int espic_clear_samples(espic_world *h, int sp) {
    WORLD(h);
    SPECIES(sp);
    int rc = ensure_ch4(w, s);
    if (rc != ESPIC_OK) return rc;
    CK(cudaMemsetAsync(s.mom, 0, NMOM * w.nn * sizeof(double), w.stream));
    return ESPIC_OK;
}

extern "C" int espic_compute_mpc(espic_world *h, int sp) {
    WORLD(h);
    SPECIES(sp);
    int rc = ensure_ch4(w, s);
    if (rc != ESPIC_OK) return rc;
    launch_mpc(w, s);
    CHECK_LAUNCH();
    return ESPIC_OK;
}

extern "C" int espic_mcc_cex(espic_world *h, int src, int tgt, double dt, const double *u, int64_t nu,
                             const int64_t *p_off, int64_t *collisions) {
    WORLD(h);
    if (src < 0 || src >= (int)w.species.size() || tgt < 0 || tgt >= (int)w.species.size())
        return fail(ESPIC_ERR_ARG, "bad species id");
    Species &s = *w.species[src], &t = *w.species[tgt];
    int rc = ensure_ch4(w, s);
    if (rc == ESPIC_OK) rc = ensure_ch4(w, t);
    if (rc != ESPIC_OK) return rc;
    if (!(dt > 0)) return fail(ESPIC_ERR_ARG, "bad time step");
    double *du = nullptr;
    int64_t *doff = nullptr;
    if (u) {
        if (!p_off || nu < 0) return fail(ESPIC_ERR_ARG, "replayed uniforms need their particle offsets");
        int64_t np = 0; /* p_off holds one entry per particle: the exact count */
        CK(cudaMemcpyAsync(&np, s.d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, w.stream));
        CK(cudaStreamSynchronize(w.stream));
        s.host_bound = np;
        if (dalloc(&du, nu > 0 ? nu : 1) != ESPIC_OK) return ESPIC_ERR_CUDA;
        if (dalloc(&doff, np > 0 ? np : 1) != ESPIC_OK) {
            cudaFree(du);
            return ESPIC_ERR_CUDA;
        }
        if (nu > 0) cudaMemcpyAsync(du, u, nu * sizeof(double), cudaMemcpyHostToDevice, w.stream);
        if (np > 0) cudaMemcpyAsync(doff, p_off, np * sizeof(int64_t), cudaMemcpyHostToDevice, w.stream);
    }
    launch_mcc(w, s, t, dt, du, nu, doff, s.mcc_ncol);
    cudaError_t e = cudaSuccess;
    if (u || collisions) e = cudaStreamSynchronize(w.stream);
    if (du) cudaFree(du);
    if (doff) cudaFree(doff);
    if (e != cudaSuccess) return fail(ESPIC_ERR_CUDA, "%s", cudaGetErrorString(e));
    CHECK_LAUNCH();
    if (collisions) {
        unsigned long long c = 0;
        CK(cudaMemcpy(&c, s.mcc_ncol, sizeof c, cudaMemcpyDeviceToHost));
        *collisions = (int64_t)c;
    }
    if (u || collisions) return take_device_errors(w);
    return ESPIC_OK;
}

extern "C" int espic_advance_ch4(espic_world *h, int sp, const double *pdt, const double *u, int64_t nu,
                                 const int64_t *p_off, int64_t *bounces) {
    WORLD(h);
    SPECIES(sp);
    if (s.form != ESPIC_FORM_FP64) return fail(ESPIC_ERR_ARG, "the ch4 push works on a species in the float64 form");
    if (s.charge != 0)
        return fail(ESPIC_ERR_ARG, "a charged species moves with espic_advance_ch4_ions");
    if (!(w.dt > 0)) return fail(ESPIC_ERR_ARG, "set the time step first");
    if (u && (!p_off || nu < 0)) return fail(ESPIC_ERR_ARG, "replayed uniforms need their particle offsets");
    if (!s.ch4_settled) {
        if (dalloc(&s.ch4_settled, 1) != ESPIC_OK || dalloc(&s.ch4_bounces, 1) != ESPIC_OK) return ESPIC_ERR_CUDA;
        CK(cudaMemsetAsync(s.ch4_settled, 0, sizeof(int64_t), w.stream));
    }
    double *dpdt = nullptr, *du = nullptr;
    int64_t *doff = nullptr;
    const bool staged = pdt || u;
    if (staged) {
        int64_t np = 0; /* pdt and p_off hold one entry per particle: the exact count */
        CK(cudaMemcpyAsync(&np, s.d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, w.stream));
        CK(cudaStreamSynchronize(w.stream));
        s.host_bound = np;
        const int64_t m = np > 0 ? np : 1;
        bool ok = true;
        if (pdt) ok = ok && dalloc(&dpdt, m) == ESPIC_OK;
        if (u) ok = ok && dalloc(&du, nu > 0 ? nu : 1) == ESPIC_OK && dalloc(&doff, m) == ESPIC_OK;
        if (!ok) {
            if (dpdt) cudaFree(dpdt);
            if (du) cudaFree(du);
            if (doff) cudaFree(doff);
            return ESPIC_ERR_CUDA;
        }
        if (pdt && np > 0) cudaMemcpyAsync(dpdt, pdt, np * sizeof(double), cudaMemcpyHostToDevice, w.stream);
        if (u && nu > 0) cudaMemcpyAsync(du, u, nu * sizeof(double), cudaMemcpyHostToDevice, w.stream);
        if (u && np > 0) cudaMemcpyAsync(doff, p_off, np * sizeof(int64_t), cudaMemcpyHostToDevice, w.stream);
    }
    {
        PhaseScope ph(w, ESPIC_PHASE_PUSH);
        launch_advance_ch4(w, s, w.dt, dpdt, du, nu, doff);
    }
    cudaError_t e = cudaSuccess;
    if (staged || bounces) e = cudaStreamSynchronize(w.stream);
    if (dpdt) cudaFree(dpdt);
    if (du) cudaFree(du);
    if (doff) cudaFree(doff);
    if (e != cudaSuccess) return fail(ESPIC_ERR_CUDA, "%s", cudaGetErrorString(e));
    CHECK_LAUNCH();
    if (bounces) {
        unsigned long long c = 0;
        CK(cudaMemcpy(&c, s.ch4_bounces, sizeof c, cudaMemcpyDeviceToHost));
        *bounces = (int64_t)c;
    }
    if (staged || bounces) return take_device_errors(w);
    return ESPIC_OK;
}

/* copies n values to a new device buffer (nothing when host is NULL) */
template <class T>
static int stage(T **d, const T *host, int64_t n, cudaStream_t st) {
    *d = nullptr;
    if (!host) return ESPIC_OK;
    if (dalloc(d, n > 0 ? n : 1) != ESPIC_OK) return ESPIC_ERR_CUDA;
    if (n > 0 && cudaMemcpyAsync(*d, host, n * sizeof(T), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return ESPIC_ERR_CUDA;
    return ESPIC_OK;
}

static int refresh_bound(World &w, Species &t) {
    int64_t c = 0;
    CK(cudaMemcpy(&c, t.d_count, sizeof c, cudaMemcpyDeviceToHost));
    t.host_bound = c;
    return ESPIC_OK;
}

extern "C" int espic_advance_ch4_ions(espic_world *h, int sp, int neutrals, int spherium, const double *pdt,
                                      const double *u, int64_t nu, const int64_t *p_off, int64_t *strikes) {
    WORLD(h);
    SPECIES(sp);
    if (s.form != ESPIC_FORM_FP64) return fail(ESPIC_ERR_ARG, "the ch4 push works on a species in the float64 form");
    if (s.charge == 0) return fail(ESPIC_ERR_ARG, "a neutral species moves with espic_advance_ch4");
    if (neutrals < 0 || neutrals >= (int)w.species.size() || spherium < 0 || spherium >= (int)w.species.size())
        return fail(ESPIC_ERR_ARG, "target species id out of range");
    if (neutrals == sp || spherium == sp)
        return fail(ESPIC_ERR_ARG, "an ion species cannot receive the particles its own strikes create");
    Species &neu = *w.species[neutrals], &sph = *w.species[spherium];
    if (neu.form != ESPIC_FORM_FP64 || sph.form != ESPIC_FORM_FP64)
        return fail(ESPIC_ERR_ARG, "the target species must be in the float64 form");
    if (!(neu.mpw0 > 0) || !(sph.mpw0 > 0) || !(s.mpw0 > 0))
        return fail(ESPIC_ERR_ARG, "the ion and target species need mpw0 > 0");
    if (!(w.dt > 0)) return fail(ESPIC_ERR_ARG, "set the time step first");
    if (u && (!p_off || nu < 0)) return fail(ESPIC_ERR_ARG, "replayed uniforms need their particle offsets");
    /* most particles one strike creates: the uniforms of one ion must fit
     * its 2^20 indices of the counter-based stream, and the counts of one
     * call an int32 scan */
    const double most = floor(s.mpw0 / neu.mpw0 + 1) + floor(0.1 * s.mpw0 / sph.mpw0 + 1);
    if (!(2 + 11 * most < (double)(1 << 20)) || !(most * (double)(s.cap + 1) < 2147483647.0))
        return fail(ESPIC_ERR_ARG, "mpw0 ratios of %g particles per strike are beyond this push", most);
    if (!s.ch4_settled) {
        if (dalloc(&s.ch4_settled, 1) != ESPIC_OK || dalloc(&s.ch4_bounces, 1) != ESPIC_OK) return ESPIC_ERR_CUDA;
        CK(cudaMemsetAsync(s.ch4_settled, 0, sizeof(int64_t), w.stream));
    }
    if (!s.ch4_cnt && dalloc(&s.ch4_cnt, 2 * (s.cap + 1) + int_scan_blocks(s.cap + 1) + 1) != ESPIC_OK)
        return ESPIC_ERR_CUDA;
    double *dpdt = nullptr, *du = nullptr;
    int64_t *doff = nullptr;
    if (pdt || u) {
        int64_t np = 0; /* pdt and p_off hold one entry per particle: the exact count */
        CK(cudaMemcpyAsync(&np, s.d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, w.stream));
        CK(cudaStreamSynchronize(w.stream));
        s.host_bound = np;
        int rc = stage(&dpdt, pdt, np, w.stream);
        if (rc == ESPIC_OK) rc = stage(&du, u, nu, w.stream);
        if (rc == ESPIC_OK) rc = stage(&doff, u ? p_off : (const int64_t *)nullptr, np, w.stream);
        if (rc != ESPIC_OK) {
            cudaFree(dpdt);
            cudaFree(du);
            cudaFree(doff);
            return fail(ESPIC_ERR_CUDA, "staging the replayed inputs failed");
        }
    }
    {
        PhaseScope ph(w, ESPIC_PHASE_PUSH);
        launch_advance_ch4_ions(w, s, neu, sph, w.dt, dpdt, du, nu, doff);
    }
    const cudaError_t e = cudaStreamSynchronize(w.stream);
    cudaFree(dpdt);
    cudaFree(du);
    cudaFree(doff);
    if (e != cudaSuccess) return fail(ESPIC_ERR_CUDA, "%s", cudaGetErrorString(e));
    CHECK_LAUNCH();
    /* the targets grew by counts known only on the device */
    if (refresh_bound(w, neu) != ESPIC_OK || refresh_bound(w, sph) != ESPIC_OK) return ESPIC_ERR_CUDA;
    if (strikes) {
        unsigned long long c = 0;
        CK(cudaMemcpy(&c, s.ch4_bounces, sizeof c, cudaMemcpyDeviceToHost));
        *strikes = (int64_t)c;
    }
    return take_device_errors(w);
}

extern "C" int espic_chemistry_ionize(espic_world *h, int neutrals, int ions, double rate, double dt,
                                      const double *u, int64_t nu, const int64_t *cell_off, int64_t *created) {
    WORLD(h);
    if (neutrals < 0 || neutrals >= (int)w.species.size() || ions < 0 || ions >= (int)w.species.size())
        return fail(ESPIC_ERR_ARG, "species id out of range");
    Species &neu = *w.species[neutrals], &ion = *w.species[ions];
    if (ion.form != ESPIC_FORM_FP64) return fail(ESPIC_ERR_ARG, "the ion species must be in the float64 form");
    if (!(ion.mpw0 > 0)) return fail(ESPIC_ERR_ARG, "the ion species needs mpw0 > 0");
    if (u && (!cell_off || nu < 0)) return fail(ESPIC_ERR_ARG, "replayed uniforms need their cell offsets");
    const int64_t ncells = (int64_t)(w.g.ni - 1) * (w.g.nj - 1) * (w.g.nk - 1);
    if (!ion.ionize_cnt && dalloc(&ion.ionize_cnt, ncells + 1 + int_scan_blocks(ncells + 1) + 1) != ESPIC_OK)
        return ESPIC_ERR_CUDA;
    double *du = nullptr;
    int64_t *doff = nullptr;
    int rc = stage(&du, u, nu, w.stream);
    if (rc == ESPIC_OK) rc = stage(&doff, u ? cell_off : (const int64_t *)nullptr, ncells, w.stream);
    if (rc != ESPIC_OK) {
        cudaFree(du);
        cudaFree(doff);
        return fail(ESPIC_ERR_CUDA, "staging the replayed inputs failed");
    }
    const uint64_t stream = (0xC6ull << 56) | ((uint64_t)(ion.id & 0xff) << 48) |
                            (ion.ionize_calls & 0xffffffffffffull);
    {
        PhaseScope ph(w, ESPIC_PHASE_INJECT);
        launch_ionize(w, neu, ion, rate, dt, du, nu, doff, ion.ionize_cnt, stream);
    }
    ion.ionize_calls++;
    const cudaError_t e = cudaStreamSynchronize(w.stream);
    cudaFree(du);
    cudaFree(doff);
    if (e != cudaSuccess) return fail(ESPIC_ERR_CUDA, "%s", cudaGetErrorString(e));
    CHECK_LAUNCH();
    int64_t c[2] = {0, 0};
    CK(cudaMemcpy(c, ion.d_count, sizeof c, cudaMemcpyDeviceToHost));
    ion.host_bound = c[0];
    if (created) *created = c[0] - c[1];
    return take_device_errors(w);
}

extern "C" int espic_species_diag(espic_world *h, int sp, double out[5]) {
    WORLD(h);
    SPECIES(sp);
    if (!out) return fail(ESPIC_ERR_ARG, "null out");
    launch_diag(w, s, w.d_small);
    CHECK_LAUNCH();
    CK(cudaMemcpyAsync(w.h_small, w.d_small, 5 * sizeof(double), cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    memcpy(out, w.h_small, 5 * sizeof(double));
    return take_device_errors(w);
}

extern "C" int espic_potential_energy(espic_world *h, double *pe) {
    WORLD(h);
    if (!pe) return fail(ESPIC_ERR_ARG, "null pe");
    launch_pe(w, w.d_small);
    CHECK_LAUNCH();
    CK(cudaMemcpyAsync(w.h_small, w.d_small, sizeof(double), cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    *pe = w.h_small[0];
    return take_device_errors(w);
}

static int diag_row_enqueue(World &w) {
    PhaseScope ph(w, ESPIC_PHASE_DIAG);
    int ns = (int)w.species.size();
    for (int i = 0; i < ns; i++) {
        Species &s = *w.species[i];
        CK(cudaMemcpyAsync(w.d_small + 6 * i, s.d_count, sizeof(int64_t), cudaMemcpyDeviceToDevice, w.stream));
        launch_diag(w, s, w.d_small + 6 * i + 1);
        CHECK_LAUNCH();
    }
    launch_pe(w, w.d_small + 6 * ns);
    CHECK_LAUNCH();
    CK(cudaMemcpyAsync(w.h_small, w.d_small, (6 * ns + 1) * sizeof(double), cudaMemcpyDeviceToHost, w.stream));
    return ESPIC_OK;
}

static int diag_row_finish(World &w, double *row) {
    CK(cudaStreamSynchronize(w.stream));
    int ns = (int)w.species.size();
    for (int i = 0; i < ns; i++) {
        int64_t n;
        memcpy(&n, w.h_small + 6 * i, sizeof n);
        w.species[i]->host_bound = n;
        row[6 * i] = (double)n;
        for (int q = 1; q < 6; q++) row[6 * i + q] = w.h_small[6 * i + q];
    }
    row[6 * ns] = w.h_small[6 * ns];
    return take_device_errors(w);
}

extern "C" int espic_diag_row(espic_world *h, double *row, int len) {
    WORLD(h);
    int ns = (int)w.species.size();
    if (!row || len < 6 * ns + 1) return fail(ESPIC_ERR_ARG, "row needs %d values", 6 * ns + 1);
    if (6 * ns + 1 > 256) return fail(ESPIC_ERR_ARG, "too many species for one row");
    int rc = diag_row_enqueue(w);
    if (rc != ESPIC_OK) return rc;
    return diag_row_finish(w, row);
}

extern "C" int espic_update_average(espic_world *h, int sp) {
    WORLD(h);
    SPECIES(sp);
    launch_update_average(w, s);
    CHECK_LAUNCH();
    return ESPIC_OK;
}

extern "C" int espic_steady_state(espic_world *h, int *steady) {
    WORLD(h);
    if (!steady) return fail(ESPIC_ERR_ARG, "null steady");
    if (w.steady) {
        *steady = 1;
        return ESPIC_OK;
    }
    int ns = (int)w.species.size();
    std::vector<double> row(6 * ns + 1);
    int rc = espic_diag_row(h, row.data(), (int)row.size());
    if (rc != ESPIC_OK) return rc;
    double tot_mass = 0, tot_mom = 0, tot_en = row[6 * ns];
    for (int i = 0; i < ns; i++) {
        tot_mass += row[6 * i + 1];
        tot_mom += fabs(row[6 * i + 4]);
        tot_en += row[6 * i + 5];
    }
    const double tol = 1e-3;
    if (fabs((tot_mass - w.last_mass) / tot_mass) < tol && fabs((tot_mom - w.last_mom) / tot_mom) < tol &&
        fabs((tot_en - w.last_en) / tot_en) < tol)
        w.steady = true;
    w.last_mass = tot_mass;
    w.last_mom = tot_mom;
    w.last_en = tot_en;
    *steady = w.steady ? 1 : 0;
    return ESPIC_OK;
}

/* ---------------------------------------------------------------- fields */
/* the ch4 species fields, allocated (zeroed) on first use */
static int ensure_ch4(World &w, Species &s) {
    if (s.ch4_on) return ESPIC_OK;
    if (s.form != 0) return fail(ESPIC_ERR_ARG, "moments and MCC work on a species in the float64 form");
    const int64_t n_cells = (int64_t)(w.g.ni - 1) * (w.g.nj - 1) * (w.g.nk - 1);
    if (dalloc(&s.mom, NMOM * w.nn) != ESPIC_OK || dalloc(&s.mom_acc, NMOM * w.nn) != ESPIC_OK ||
        dalloc(&s.mom_scale, 2 * NMOM) != ESPIC_OK || dalloc(&s.mom_bound, NMOM) != ESPIC_OK ||
        dalloc(&s.gvel, 3 * w.nn) != ESPIC_OK || dalloc(&s.gtemp, w.nn) != ESPIC_OK ||
        dalloc(&s.mpc, n_cells) != ESPIC_OK || dalloc(&s.mcc_ncol, 1) != ESPIC_OK)
        return ESPIC_ERR_CUDA;
    CK(cudaMemsetAsync(s.mom, 0, NMOM * w.nn * sizeof(double), w.stream));
    CK(cudaMemsetAsync(s.mom_acc, 0, NMOM * w.nn * sizeof(unsigned long long), w.stream));
    CK(cudaMemsetAsync(s.gvel, 0, 3 * w.nn * sizeof(double), w.stream));
    CK(cudaMemsetAsync(s.gtemp, 0, w.nn * sizeof(double), w.stream));
    CK(cudaMemsetAsync(s.mpc, 0, n_cells * sizeof(double), w.stream));
    s.ch4_on = true;
    return ESPIC_OK;
}

static int field_ptr(World &w, int field, int sp, double **p, int64_t *count) {
    switch (field) {
        case ESPIC_FIELD_PHI: *p = w.phi; *count = w.nn; return ESPIC_OK;
        case ESPIC_FIELD_RHO: *p = w.rho; *count = w.nn; return ESPIC_OK;
        case ESPIC_FIELD_NODE_VOL: *p = w.vol; *count = w.nn; return ESPIC_OK;
        case ESPIC_FIELD_EF:
            ensure_ef64(w); /* the float64 field of a mixed-form world is completed on demand */
            *p = w.ef;
            *count = 3 * w.nn;
            return ESPIC_OK;
        case ESPIC_FIELD_DEN:
        case ESPIC_FIELD_DEN_AVE:
            if (sp < 0 || sp >= (int)w.species.size()) return fail(ESPIC_ERR_ARG, "bad species id");
            *p = field == ESPIC_FIELD_DEN ? w.species[sp]->den : w.species[sp]->den_ave;
            *count = w.nn;
            return ESPIC_OK;
        case ESPIC_FIELD_VEL:
        case ESPIC_FIELD_TEMP:
        case ESPIC_FIELD_MPC:
        case ESPIC_FIELD_MOMENTS: {
            if (sp < 0 || sp >= (int)w.species.size()) return fail(ESPIC_ERR_ARG, "bad species id");
            Species &s = *w.species[sp];
            int rc = ensure_ch4(w, s);
            if (rc != ESPIC_OK) return rc;
            const int64_t n_cells = (int64_t)(w.g.ni - 1) * (w.g.nj - 1) * (w.g.nk - 1);
            if (field == ESPIC_FIELD_VEL) *p = s.gvel, *count = 3 * w.nn;
            if (field == ESPIC_FIELD_TEMP) *p = s.gtemp, *count = w.nn;
            if (field == ESPIC_FIELD_MPC) *p = s.mpc, *count = n_cells;
            if (field == ESPIC_FIELD_MOMENTS) *p = s.mom, *count = NMOM * w.nn;
            return ESPIC_OK;
        }
        default:
            return fail(ESPIC_ERR_ARG, "unknown field %d", field);
    }
}

extern "C" int espic_field_read(espic_world *h, int field, int sp, double *host, int64_t n) {
    WORLD(h);
    if (!host) return fail(ESPIC_ERR_ARG, "null host buffer");
    if (field == ESPIC_FIELD_OBJECT_ID) {
        if (n < w.nn) return fail(ESPIC_ERR_ARG, "buffer too small");
        std::vector<int32_t> tmp(w.nn);
        CK(cudaMemcpyAsync(tmp.data(), w.obj, w.nn * sizeof(int32_t), cudaMemcpyDeviceToHost, w.stream));
        CK(cudaStreamSynchronize(w.stream));
        for (int64_t i = 0; i < w.nn; i++) host[i] = tmp[i];
        return ESPIC_OK;
    }
    double *p;
    int64_t cnt;
    int rc = field_ptr(w, field, sp, &p, &cnt);
    if (rc != ESPIC_OK) return rc;
    if (n < cnt) return fail(ESPIC_ERR_ARG, "buffer holds %lld of %lld values", (long long)n, (long long)cnt);
    CK(cudaMemcpyAsync(host, p, cnt * sizeof(double), cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    return take_device_errors(w);
}

extern "C" int espic_field_write(espic_world *h, int field, int sp, const double *host, int64_t n) {
    WORLD(h);
    if (!host) return fail(ESPIC_ERR_ARG, "null host buffer");
    if (field == ESPIC_FIELD_OBJECT_ID) {
        if (n < w.nn) return fail(ESPIC_ERR_ARG, "buffer too small");
        std::vector<int32_t> tmp(w.nn);
        for (int64_t i = 0; i < w.nn; i++) tmp[i] = (int32_t)host[i];
        CK(cudaMemcpyAsync(w.obj, tmp.data(), w.nn * sizeof(int32_t), cudaMemcpyHostToDevice, w.stream));
        CK(cudaStreamSynchronize(w.stream));
        w.targets_valid = false;
        w.pcg_codes_valid = false;
        w.phi_prev_valid = false;
        return ESPIC_OK;
    }
    if (field == ESPIC_FIELD_MOMENTS) return fail(ESPIC_ERR_ARG, "the sampled sums are read only");
    double *p;
    int64_t cnt;
    int rc = field_ptr(w, field, sp, &p, &cnt);
    if (rc != ESPIC_OK) return rc;
    if (n < cnt) return fail(ESPIC_ERR_ARG, "buffer holds %lld of %lld values", (long long)n, (long long)cnt);
    CK(cudaMemcpyAsync(p, host, cnt * sizeof(double), cudaMemcpyHostToDevice, w.stream));
    if (field == ESPIC_FIELD_EF) {
        launch_ef4(w);
        w.ef64_valid = true;
    }
    /* a written field or volume: the cached energy sum no longer applies */
    if (field == ESPIC_FIELD_EF || field == ESPIC_FIELD_NODE_VOL) w.pe_parts = 0;
    if (field == ESPIC_FIELD_NODE_VOL) launch_inv_vol(w);
    if (field == ESPIC_FIELD_PHI) w.phi_prev_valid = false;
    if (field == ESPIC_FIELD_RHO) w.rho_version++;
    CHECK_LAUNCH();
    CK(cudaStreamSynchronize(w.stream));
    return ESPIC_OK;
}

/* ---------------------------------------------------------------- output snapshots */
extern "C" int espic_snapshot_begin(espic_world *h, int64_t *ticket) {
    WORLD(h);
    if (!ticket) return fail(ESPIC_ERR_ARG, "null ticket");
    const int ns = (int)w.species.size() < 8 ? (int)w.species.size() : 8;
    const size_t count = (size_t)(7 + 2 * ns) * w.nn;
    if (!w.snap_stream) CK(cudaStreamCreateWithFlags(&w.snap_stream, cudaStreamNonBlocking));
    World::Snapshot &sn = w.snap[w.snap_next & 1];
    if (sn.copied) CK(cudaEventSynchronize(sn.copied)); /* the slot's previous copy is done */
    if (sn.count < count) {
        if (sn.dev) cudaFree(sn.dev);
        if (sn.host) cudaFreeHost(sn.host);
        sn.dev = nullptr;
        sn.host = nullptr;
        sn.count = 0;
        CK(cudaMalloc(&sn.dev, count * sizeof(double)));
        CK(cudaMallocHost(&sn.host, count * sizeof(double)));
        sn.count = count;
    }
    if (!sn.packed) CK(cudaEventCreateWithFlags(&sn.packed, cudaEventDisableTiming));
    if (!sn.copied) CK(cudaEventCreateWithFlags(&sn.copied, cudaEventDisableTiming));
    launch_snapshot(w, sn.dev);
    CHECK_LAUNCH();
    CK(cudaEventRecord(sn.packed, w.stream));
    CK(cudaStreamWaitEvent(w.snap_stream, sn.packed, 0));
    CK(cudaMemcpyAsync(sn.host, sn.dev, count * sizeof(double), cudaMemcpyDeviceToHost, w.snap_stream));
    CK(cudaEventRecord(sn.copied, w.snap_stream));
    sn.ticket = w.snap_next++;
    *ticket = sn.ticket;
    return ESPIC_OK;
}

extern "C" int espic_snapshot_wait(espic_world *h, int64_t ticket, const double **host, int64_t *count) {
    if (!h) return fail(ESPIC_ERR_ARG, "null world handle");
    World &w = h->w;
    World::Snapshot &sn = w.snap[ticket & 1];
    if (ticket < 0 || sn.ticket != ticket) return fail(ESPIC_ERR_STATE, "snapshot %lld is no longer held", (long long)ticket);
    if (cudaSetDevice(w.device) != cudaSuccess) return fail(ESPIC_ERR_CUDA, "cudaSetDevice failed");
    CK(cudaEventSynchronize(sn.copied));
    if (host) *host = sn.host;
    if (count) *count = (int64_t)sn.count;
    return ESPIC_OK;
}

/* ---------------------------------------------------------------- the whole step */
extern "C" int espic_step(espic_world *h, int sort_every, double *row, int len) {
    WORLD(h);
    int ns = (int)w.species.size();
    if (row && len < 6 * ns + 1) return fail(ESPIC_ERR_ARG, "row needs %d values", 6 * ns + 1);
    int rc;
    for (int src = 0; src < (int)w.sources.size(); src++)
        if ((rc = espic_source_sample(h, src)) != ESPIC_OK) return rc;
    for (Species *s : w.species) {
        if (s->form == ESPIC_FORM_MIXED && sort_every > 0 && (w.step_count % sort_every) == 0) {
            PhaseScope ph(w, ESPIC_PHASE_SORT);
            launch_sort_mixed(w, *s);
            CHECK_LAUNCH();
        }
        if (!(s->weight_bound > 0)) set_weight_bound(*s, 1.0);
        if ((rc = push_one(w, *s, true)) != ESPIC_OK) return rc;
    }
    {
        PhaseScope ph(w, ESPIC_PHASE_DENSITY);
        launch_charge(w);
        w.rho_version++;
    }
    CHECK_LAUNCH();
    if ((rc = enqueue_solve(w)) != ESPIC_OK) return rc;
    {
        PhaseScope ph(w, ESPIC_PHASE_EFIELD);
        launch_efield(w, false);
    }
    CHECK_LAUNCH();
    w.step_count++;
    if (!row) return ESPIC_OK;
    if ((rc = diag_row_enqueue(w)) != ESPIC_OK) return rc;
    return diag_row_finish(w, row);
}

/* ---------------------------------------------------------------- measurement */
extern "C" int espic_profile(espic_world *h, int enable) {
    WORLD(h);
    prof_collect(w);
    w.prof = enable != 0;
    for (int i = 0; i < ESPIC_NPHASES; i++) {
        w.prof_ms[i] = 0;
        w.prof_n[i] = 0;
    }
    return ESPIC_OK;
}

extern "C" int espic_profile_read(espic_world *h, double ms[ESPIC_NPHASES], int64_t count[ESPIC_NPHASES],
                                  int64_t *launches) {
    WORLD(h);
    prof_collect(w);
    CK(cudaStreamSynchronize(w.stream));
    for (int i = 0; i < ESPIC_NPHASES; i++) {
        if (ms) ms[i] = w.prof_ms[i];
        if (count) count[i] = w.prof_n[i];
    }
    if (launches) *launches = w.nlaunch;
    return ESPIC_OK;
}

extern "C" int espic_solver_totals(espic_world *h, int64_t *solves, int64_t *outer, int64_t *inner) {
    WORLD(h);
    SolveStatus st;
    CK(cudaMemcpyAsync(&st, w.d_status, sizeof st, cudaMemcpyDeviceToHost, w.stream));
    CK(cudaStreamSynchronize(w.stream));
    if (solves) *solves = st.solves;
    if (outer) *outer = st.outer_total;
    if (inner) *inner = st.inner_total;
    return ESPIC_OK;
}
