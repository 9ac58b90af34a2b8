// sample.cu -- batched stochastic forward traceback of the 2D pair HMM
// (dp/hmm.py:2043-2101 sample_traceback_2d).
//
// Two launches:
//   fwdlog_kernel  one CTA per pair sweeps the anti-diagonals in float64 log
//                  space and keeps the whole forward table F (Lx+1)(Ly+1)N,
//                  with the reference's arithmetic: F[i][j][k] = logsumexp_s
//                  (F[pred(k)][s] + logchi[s][k]) + logemit_k, NEG_INF (-1e30)
//                  summed like any other number; the log-likelihood is
//                  logsumexp_s F[Lx][Ly][s] + logchi[s][E];
//   sample_kernel  one thread per (pair, sample) walks back from (Lx, Ly): the
//                  final state with probability proportional to
//                  exp(F[Lx][Ly][s] + logchi[s][E]), then at each cell the
//                  predecessor cell fixed by the current state's type (M: i-1,
//                  j-1; I: j-1; D: i-1) and its state with probability
//                  proportional to exp(F[pred][s] + logchi[s][k]), until (0, 0);
//                  the path is written from (0, 0, S) on, as the reference
//                  returns it.
//
// Random numbers: a counter-based stream, no state between launches.  Draw n
// of sample s of pair p is u = top 53 bits of mix(mix(seed + K (p * 2^32 +
// s)) + K n) / 2^53, mix the SplitMix64 output function (Steele, Lea and
// Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014) and K
// its golden-ratio increment.  A state is chosen as the first index whose
// running sum of exp(score - max) exceeds u times the total, the inverse-CDF
// rule; the reference draws with jax.random.choice (other numbers, the same
// distribution).
#include "pairhmm.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

extern "C" __attribute__((visibility("hidden"))) void phmm_internal_set_error(const char *msg);

namespace smp {

constexpr int NT = 256;
constexpr int ST = 128;   // sampler threads per CTA
constexpr int MAXN = 64;
constexpr double NEG = -1e30;   // the reference's NEG_INF (dp/hmm.py:108)
constexpr int TS = 0, TM = 1, TI = 2, TD = 3;
constexpr unsigned long long GOLDEN = 0x9e3779b97f4a7c15ULL;

struct Meta {
    int64_t x_off, y_off, f_off, path_off;   // path_off: first triple of the pair's sample block
    int32_t Lx, Ly;
};

struct Desc {
    int N, G, e_idx, s_idx;
    int8_t type[MAXN];
    int8_t group[MAXN];
};

__host__ __device__ inline unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__device__ inline double uniform(unsigned long long stream, unsigned long long n) {
    return (double)(mix64(stream + GOLDEN * n) >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void __launch_bounds__(NT)
fwdlog_kernel(const __grid_constant__ Desc d, const Meta *__restrict__ meta, const uint8_t *__restrict__ res,
              const double *__restrict__ lchi_all, int chi_pp, const double *__restrict__ lM,
              const double *__restrict__ lI, const double *__restrict__ lD, int emit_pp, double *__restrict__ F,
              double *__restrict__ ll_out, int32_t *__restrict__ status) {
    extern __shared__ double lchi[];   // [N][N]
    const int p = blockIdx.x, tid = threadIdx.x;
    const Meta m = meta[p];
    const int N = d.N, G = d.G;
    const double *lc = lchi_all + (chi_pp ? (int64_t)p * N * N : 0);
    for (int idx = tid; idx < N * N; idx += NT) lchi[idx] = lc[idx];
    const double *eM = lM + (emit_pp ? (int64_t)p * G * 441 : 0);
    const double *eI = lI + (emit_pp ? (int64_t)p * G * 21 : 0);
    const double *eD = lD + (emit_pp ? (int64_t)p * G * 21 : 0);
    const int Lx = m.Lx, Ly = m.Ly;
    double *Fp = F + m.f_off;
    __syncthreads();
    for (int dd = 0; dd <= Lx + Ly; ++dd) {
        const int i_lo = max(0, dd - Ly), i_hi = min(dd, Lx);
        const int ncell = i_hi - i_lo + 1;
        for (int item = tid; item < ncell * N; item += NT) {
            const int i = i_lo + item / N, k = item % N, j = dd - i;
            double *out = Fp + ((int64_t)i * (Ly + 1) + j) * N + k;
            if (dd == 0) {
                *out = k == d.s_idx ? 0.0 : NEG;
                continue;
            }
            const int st = d.type[k];
            const double *pred = nullptr;
            if (st == TM && i > 0 && j > 0) pred = Fp + ((int64_t)(i - 1) * (Ly + 1) + j - 1) * N;
            else if (st == TI && j > 0) pred = Fp + ((int64_t)i * (Ly + 1) + j - 1) * N;
            else if (st == TD && i > 0) pred = Fp + ((int64_t)(i - 1) * (Ly + 1) + j) * N;
            if (!pred) {
                *out = NEG;
                continue;
            }
            double mx = pred[0] + lchi[k];
            for (int s = 1; s < N; ++s) mx = fmax(mx, pred[s] + lchi[s * N + k]);
            double sum = 0.0;
            for (int s = 0; s < N; ++s) sum += exp(pred[s] + lchi[s * N + k] - mx);
            const int xa = i > 0 ? min((int)res[m.x_off + i - 1], 20) : 0;
            const int yb = j > 0 ? min((int)res[m.y_off + j - 1], 20) : 0;
            const int g = d.group[k];
            double e;
            if (st == TM) e = eM[g * 441 + xa * 21 + yb];
            else if (st == TI) e = eI[g * 21 + yb];
            else e = eD[g * 21 + xa];
            *out = mx + log(sum) + e;
        }
        __syncthreads();
    }
    if (tid == 0) {
        const double *last = Fp + ((int64_t)Lx * (Ly + 1) + Ly) * N;
        double mx = last[0] + lchi[d.e_idx];
        for (int s = 1; s < N; ++s) mx = fmax(mx, last[s] + lchi[s * N + d.e_idx]);
        double sum = 0.0;
        for (int s = 0; s < N; ++s) sum += exp(last[s] + lchi[s * N + d.e_idx] - mx);
        const double ll = mx + log(sum);
        ll_out[p] = ll;
        if (!(ll > -1e29)) atomicOr(status + p, PHMM_ST_ZERO_LL);
    }
}

// Inverse-CDF draw over scores v[0..N) (probabilities exp(v - logsumexp v)).
__device__ inline int draw(const double *v, int N, double u) {
    double mx = v[0];
    for (int s = 1; s < N; ++s) mx = fmax(mx, v[s]);
    double tot = 0.0;
    for (int s = 0; s < N; ++s) tot += exp(v[s] - mx);
    const double target = u * tot;
    double cum = 0.0;
    for (int s = 0; s < N; ++s) {
        cum += exp(v[s] - mx);
        if (cum > target) return s;
    }
    return N - 1;
}

__global__ void __launch_bounds__(ST)
sample_kernel(const __grid_constant__ Desc d, const Meta *__restrict__ meta, const double *__restrict__ lchi_all,
              int chi_pp, const double *__restrict__ F, int n_samples, unsigned long long seed,
              int32_t *__restrict__ paths, int32_t *__restrict__ path_len) {
    const int p = blockIdx.x, smp = blockIdx.y * ST + threadIdx.x;
    if (smp >= n_samples) return;
    const Meta m = meta[p];
    const int N = d.N, Lx = m.Lx, Ly = m.Ly;
    const double *lc = lchi_all + (chi_pp ? (int64_t)p * N * N : 0);
    const double *Fp = F + m.f_off;
    const int slot = Lx + Ly + 1;
    int32_t *pp = paths + 3 * (m.path_off + (int64_t)smp * slot);
    const unsigned long long stream = mix64(seed + GOLDEN * (((unsigned long long)p << 32) | (unsigned)smp));
    unsigned long long n = 0;
    double v[MAXN];
    const double *last = Fp + ((int64_t)Lx * (Ly + 1) + Ly) * N;
    for (int s = 0; s < N; ++s) v[s] = last[s] + lc[s * N + d.e_idx];
    int ck = draw(v, N, uniform(stream, n++));
    int ci = Lx, cj = Ly, len = 0;
    while ((ci > 0 || cj > 0) && len < Lx + Ly) {
        pp[3 * len] = ci; pp[3 * len + 1] = cj; pp[3 * len + 2] = ck;
        ++len;
        const int st = d.type[ck];
        int pi_, pj_;
        if (st == TM && ci > 0 && cj > 0) { pi_ = ci - 1; pj_ = cj - 1; }
        else if (st == TI && cj > 0) { pi_ = ci; pj_ = cj - 1; }
        else if (st == TD && ci > 0) { pi_ = ci - 1; pj_ = cj; }
        else break;
        const double *pr = Fp + ((int64_t)pi_ * (Ly + 1) + pj_) * N;
        for (int s = 0; s < N; ++s) v[s] = pr[s] + lc[s * N + ck];
        ck = draw(v, N, uniform(stream, n++));
        ci = pi_;
        cj = pj_;
    }
    pp[3 * len] = 0; pp[3 * len + 1] = 0; pp[3 * len + 2] = d.s_idx;
    ++len;
    for (int a = 0, b = len - 1; a < b; ++a, --b)
        for (int c = 0; c < 3; ++c) {
            const int32_t t = pp[3 * a + c];
            pp[3 * a + c] = pp[3 * b + c];
            pp[3 * b + c] = t;
        }
    path_len[(int64_t)p * n_samples + smp] = len;
}

}  // namespace smp

static int smp_fail(int code, const char *msg) {
    phmm_internal_set_error(msg);
    return code;
}

static size_t smp_align(size_t v) { return (v + 255) & ~(size_t)255; }

struct SmpLayout {
    std::vector<smp::Meta> meta;
    size_t o_F, total;
};

static int smp_layout(const phmm_batch *b, int N, int n_samples, SmpLayout &L) {
    const int P = b->n_pairs;
    L.meta.resize(P);
    int64_t f = 0, pth = 0;
    for (int p = 0; p < P; ++p) {
        const int Lx = b->Lx_host[p], Ly = b->Ly_host[p];
        if (Lx < 0 || Ly < 0) return smp_fail(PHMM_E_ARG, "phmm_sample_paths: negative length");
        L.meta[p] = smp::Meta{b->x_off_host[p], b->y_off_host[p], f, pth, Lx, Ly};
        f += (int64_t)(Lx + 1) * (Ly + 1) * N;
        pth += (int64_t)n_samples * (Lx + Ly + 1);
    }
    L.o_F = smp_align(sizeof(smp::Meta) * (size_t)P);
    L.total = smp_align(L.o_F + sizeof(double) * (size_t)f);
    return PHMM_OK;
}

extern "C" int phmm_sample_workspace_bytes(const phmm_model_desc *model, const phmm_batch *batch, size_t *bytes) {
    if (!model || !batch || !bytes) return smp_fail(PHMM_E_ARG, "phmm_sample_workspace_bytes: null argument");
    *bytes = 0;
    if (batch->n_pairs <= 0) return PHMM_OK;
    if (!batch->Lx_host || !batch->Ly_host || !batch->x_off_host || !batch->y_off_host)
        return smp_fail(PHMM_E_ARG, "phmm_sample_paths: null host length or offset array");
    SmpLayout L;
    int rc = smp_layout(batch, model->n_states, 0, L);
    if (rc) return rc;
    *bytes = L.total;
    return PHMM_OK;
}

extern "C" int phmm_sample_paths(const phmm_model_desc *model, const phmm_batch *batch, const double *log_chi,
                                 const double *log_emit_M, const double *log_emit_I, const double *log_emit_D,
                                 int32_t n_samples, uint64_t seed, void *workspace, size_t workspace_bytes,
                                 double *ll_out, int32_t *paths, int32_t *path_len, int32_t *status_out,
                                 void *stream) {
    using namespace smp;
    if (!model || !model->state_types || !model->state_group || !batch)
        return smp_fail(PHMM_E_ARG, "phmm_sample_paths: bad model description or batch");
    const int N = model->n_states, G = model->n_groups, P = batch->n_pairs;
    if (N < 2 || N > MAXN) return smp_fail(PHMM_E_ARG, "phmm_sample_paths: n_states must be in 2..64");
    if (G < 1) return smp_fail(PHMM_E_ARG, "phmm_sample_paths: n_groups must be positive");
    if (P < 0 || n_samples < 0) return smp_fail(PHMM_E_ARG, "phmm_sample_paths: negative n_pairs or n_samples");
    if (P == 0) return PHMM_OK;
    if (n_samples > 65535 * ST)
        return smp_fail(PHMM_E_ARG, "phmm_sample_paths: at most 8388480 samples per pair in one call");
    if (!batch->Lx_host || !batch->Ly_host || !batch->x_off_host || !batch->y_off_host || !batch->residues ||
        !log_chi || !log_emit_M || !log_emit_I || !log_emit_D || !workspace || !ll_out || !status_out ||
        (n_samples > 0 && (!paths || !path_len)))
        return smp_fail(PHMM_E_ARG, "phmm_sample_paths: null pointer");
    if ((uintptr_t)workspace & 255)
        return smp_fail(PHMM_E_ARG, "phmm_sample_paths: workspace must be 256-byte aligned");
    Desc d;
    std::memset(&d, 0, sizeof(d));
    d.N = N;
    d.G = G;
    d.e_idx = -1;
    d.s_idx = 0;
    for (int s = 0; s < N; ++s) {
        d.type[s] = model->state_types[s];
        d.group[s] = (int8_t)std::max(0, std::min(G - 1, (int)model->state_group[s]));
        if (d.type[s] == 4 && d.e_idx < 0) d.e_idx = s;
    }
    if (d.type[0] != TS || d.e_idx < 0)
        return smp_fail(PHMM_E_ARG, "phmm_sample_paths: state 0 must be S and one state E");
    SmpLayout L;
    int rc = smp_layout(batch, N, n_samples, L);
    if (rc) return rc;
    if (workspace_bytes < L.total) return smp_fail(PHMM_E_ARG, "phmm_sample_paths: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    cudaError_t e = cudaMemcpyAsync(ws, L.meta.data(), sizeof(Meta) * P, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(status_out, 0, sizeof(int32_t) * P, st);
    if (e != cudaSuccess) return smp_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    const size_t smem = sizeof(double) * N * N;
    e = cudaFuncSetAttribute(fwdlog_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return smp_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    fwdlog_kernel<<<P, NT, smem, st>>>(d, (const Meta *)ws, batch->residues, log_chi, batch->chi_per_pair,
                                      log_emit_M, log_emit_I, log_emit_D, batch->emit_per_pair,
                                      (double *)(ws + L.o_F), ll_out, status_out);
    if (n_samples > 0) {
        dim3 grid(P, (n_samples + ST - 1) / ST);
        sample_kernel<<<grid, ST, 0, st>>>(d, (const Meta *)ws, log_chi, batch->chi_per_pair,
                                           (const double *)(ws + L.o_F), n_samples, (unsigned long long)seed,
                                           paths, path_len);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return smp_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}
