/*
 * noalloc.cu -- espic_deposit_noalloc: the fixed-point CIC charge deposit of
 * Species::computeNumberDensity for callers that may not allocate device
 * memory (see include/espic.h for who they are).
 *
 * The deposit needs an int64 accumulator the size of the node grid.  Here it
 * is a file-scope __device__ array of ESPIC_NOALLOC_MAX_NODES entries
 * (8 MiB), so the call itself allocates nothing: every GPU that loads
 * libespic holds those 8 MiB until the process exits.  Host code may not
 * hand the array's name to a kernel (on the host it is only a stand-in), so
 * the device address is fetched with cudaGetSymbolAddress once per device,
 * with that device current, on the first call made on it; the kernels
 * receive that address.  All calls share the one array and leave their sums
 * in it, so each call clears the part it uses first, and calls that overlap
 * on the GPU (different streams, or different host threads on one device)
 * race on it.  Particles the fixed-point sum cannot take (a weight beyond
 * weight_bound, a non-finite position) are skipped and reported in the
 * caller's flag word, the counterpart of the allocating path's
 * ESPIC_ERR_FIXED and ESPIC_ERR_NONFINITE.
 *
 * The arithmetic is the float64 deposit of k_fp64.cu: corner weights
 * value*(1-di)*(1-dj)*(1-dk) in the reference's corner order (Field_::scatter,
 * ch2/Field.h:164-183), each rounded once to a count of 1/fx, then
 * den = count/fx / node_volume (World::computeNodeVolumes,
 * ch2/World.cpp:58-69).  Built with -fmad=false like k_fp64.cu.
 */
#include <math.h>
#include <stdio.h>

#include <mutex>

#include "espic.h"

namespace {

__device__ __align__(256) unsigned long long g_noalloc_acc[ESPIC_NOALLOC_MAX_NODES];

struct NaGeo {
    int ni, nj, nk;
    double x0[3], dh[3];
};

__device__ __forceinline__ int na_clamp(int i, int n) { return i < 0 ? 0 : (i > n - 2 ? n - 2 : i); }

__global__ void k_na_clear(unsigned long long *acc, int64_t nn, int *flags) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u < nn) acc[u] = 0ull;
    if (u == 0 && flags) *flags = 0;
}

/* A particle whose position is not finite, or whose weight is not within
 * [-weight_bound, weight_bound] (so that its corner counts could wrap the
 * int64 sums), deposits nothing and sets a bit of *flags. */
__global__ void k_na_deposit(NaGeo g, const double *__restrict__ P, int64_t stride, int64_t n, double fx,
                             double weight_bound, unsigned long long *acc, int *flags) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    double lc[3];
    for (int d = 0; d < 3; d++) lc[d] = (P[d * stride + p] - g.x0[d]) / g.dh[d];
    double value = P[6 * stride + p];
    const bool finite = isfinite(lc[0]) && isfinite(lc[1]) && isfinite(lc[2]);
    const bool in_range = fabs(value) <= weight_bound; /* false for NaN */
    if (!(finite && in_range)) {
        if (flags) atomicOr(flags, (finite ? 0 : ESPIC_NOALLOC_NONFINITE) | (in_range ? 0 : ESPIC_NOALLOC_RANGE));
        return;
    }
    int i = na_clamp((int)lc[0], g.ni), j = na_clamp((int)lc[1], g.nj), k = na_clamp((int)lc[2], g.nk);
    double di = lc[0] - i, dj = lc[1] - j, dk = lc[2] - k;
    int64_t n0 = ((int64_t)k * g.nj + j) * g.ni + i;
    int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    double w[8];
    w[0] = value * (1 - di) * (1 - dj) * (1 - dk);
    w[1] = value * (di) * (1 - dj) * (1 - dk);
    w[2] = value * (di) * (dj) * (1 - dk);
    w[3] = value * (1 - di) * (dj) * (1 - dk);
    w[4] = value * (1 - di) * (1 - dj) * (dk);
    w[5] = value * (di) * (1 - dj) * (dk);
    w[6] = value * (di) * (dj) * (dk);
    w[7] = value * (1 - di) * (dj) * (dk);
    int64_t idx[8] = {n0, n0 + 1, n0 + 1 + sy, n0 + sy, n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
    for (int m = 0; m < 8; m++) {
        long long q = __double2ll_rn(w[m] * fx);
        if (q != 0) atomicAdd(acc + idx[m], (unsigned long long)q);
    }
}

__global__ void k_na_density(NaGeo g, const unsigned long long *__restrict__ acc, double unit, double *den) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    if (u >= nn) return;
    int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / ((int64_t)g.ni * g.nj));
    double V = g.dh[0] * g.dh[1] * g.dh[2];
    if (i == 0 || i == g.ni - 1) V *= 0.5;
    if (j == 0 || j == g.nj - 1) V *= 0.5;
    if (k == 0 || k == g.nk - 1) V *= 0.5;
    double d = __ll2double_rn((long long)acc[u]) * unit;
    den[u] = (V != 0) ? d / V : 0.0;
}

std::mutex g_na_mutex;
constexpr int NA_MAX_DEVICES = 64;
void *g_na_addr[NA_MAX_DEVICES] = {nullptr};

}  // namespace

int espic_internal_fail(int code, const char *msg);

/* The device address of g_noalloc_acc for the current device, looked up once
 * per device with that device current. */
static int na_scratch(unsigned long long **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return espic_internal_fail(ESPIC_ERR_CUDA, "espic_deposit_noalloc: no current device");
    if (dev < 0 || dev >= NA_MAX_DEVICES)
        return espic_internal_fail(ESPIC_ERR_ARG, "espic_deposit_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_acc);
        if (e != cudaSuccess || !p) {
            char buf[256];
            snprintf(buf, sizeof buf, "espic_deposit_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return espic_internal_fail(ESPIC_ERR_CUDA, buf);
        }
        g_na_addr[dev] = p;
    }
    *out = (unsigned long long *)g_na_addr[dev];
    return ESPIC_OK;
}

extern "C" int espic_deposit_noalloc(const double *d_P, int64_t stride, int64_t n, int ni, int nj, int nk,
                                     const double x0[3], const double xm[3], double weight_bound, double *d_den,
                                     int *d_flags, void *stream) {
    if (!x0 || !xm || !d_den || (n > 0 && !d_P))
        return espic_internal_fail(ESPIC_ERR_ARG, "espic_deposit_noalloc: null argument");
    if (ni < 3 || nj < 3 || nk < 3)
        return espic_internal_fail(ESPIC_ERR_ARG, "espic_deposit_noalloc: need at least 3 nodes per axis");
    /* bound each factor before multiplying, so that no product can wrap */
    if (ni > ESPIC_NOALLOC_MAX_NODES || nj > ESPIC_NOALLOC_MAX_NODES || nk > ESPIC_NOALLOC_MAX_NODES ||
        (int64_t)ni * nj > ESPIC_NOALLOC_MAX_NODES / nk) {
        char buf[240];
        snprintf(buf, sizeof buf,
                 "espic_deposit_noalloc: a %d x %d x %d grid exceeds its fixed scratch of %d nodes; use "
                 "espic_deposit",
                 ni, nj, nk, ESPIC_NOALLOC_MAX_NODES);
        return espic_internal_fail(ESPIC_ERR_ARG, buf);
    }
    const int64_t nn = (int64_t)ni * nj * nk;
    if (n < 0 || stride < n) return espic_internal_fail(ESPIC_ERR_ARG, "espic_deposit_noalloc: bad particle count");
    if (!(weight_bound > 0)) return espic_internal_fail(ESPIC_ERR_ARG, "espic_deposit_noalloc: weight_bound <= 0");
    for (int d = 0; d < 3; d++)
        if (!(xm[d] > x0[d])) return espic_internal_fail(ESPIC_ERR_ARG, "espic_deposit_noalloc: xm <= x0");
    unsigned long long *acc = nullptr;
    int rc = na_scratch(&acc);
    if (rc != ESPIC_OK) return rc;
    NaGeo g;
    g.ni = ni;
    g.nj = nj;
    g.nk = nk;
    int nn3[3] = {ni, nj, nk};
    for (int d = 0; d < 3; d++) {
        g.x0[d] = x0[d];
        g.dh[d] = (xm[d] - x0[d]) / (nn3[d] - 1);
    }
    /* the fixed-point scale of a species of capacity n with this weight bound */
    int64_t cap = n < 1 ? 1 : n;
    double lim = ldexp(1.0, 62) / ((double)cap * weight_bound);
    int ex;
    frexp(lim, &ex);
    int S = ex - 1 > 52 ? 52 : ex - 1;
    double fx = ldexp(1.0, S);
    cudaStream_t st = (cudaStream_t)stream;
    k_na_clear<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(acc, nn, d_flags);
    if (n > 0)
        k_na_deposit<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, d_P, stride, n, fx, weight_bound, acc, d_flags);
    k_na_density<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(g, acc, 1.0 / fx, d_den);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char buf[200];
        snprintf(buf, sizeof buf, "espic_deposit_noalloc: launch: %s", cudaGetErrorString(e));
        return espic_internal_fail(ESPIC_ERR_CUDA, buf);
    }
    return ESPIC_OK;
}
