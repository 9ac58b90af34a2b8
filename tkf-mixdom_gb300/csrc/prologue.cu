// prologue.cu -- device builders of the MixDom2 E-step inputs, per pair time t.
//
// The reference builds these inside its jitted E-step for every pair
// (train/likelihood.py:143-373 calls models/mixdom.py:104-423 for the
// collapsed transition matrix chi, core/ctmc.py:31-60 / train/vjp.py:463-510
// for P_c(t) = expm(t Q_c), and dp/hmm.py:673-783 for the per-class mixture
// emission tables).  Here three launches do the same for a whole batch:
//
//   chi_kernel     one CTA per pair: TKF91 matrices of the main level and of
//                  every domain (core/bdi.py:40-99 with its lambda ~ mu
//                  branches), the null-domain closure (I - T_nn)^-1 applied
//                  from the left by T_Nnull (one Gauss-Jordan solve with five
//                  right-hand sides), T_exit_k, the effective 5x5 T, and the
//                  N x N collapsed matrix written as float32;
//   expm_kernel    one CTA per (pair, class): Q_c from (S_exch, pi), then
//                  exp(t Q_c) by scaling and squaring with the degree-13 Pade
//                  approximant of Higham, "The scaling and squaring method
//                  for the matrix exponential revisited", SIAM J. Matrix
//                  Anal. Appl. 26 (2005), Algorithm 2.3 (the method
//                  jax.scipy.linalg.expm implements), float64;
//   tables_kernel  one CTA per pair: EM[g][a][b] = sum_c w[g][c]
//                  max(pi_c[a],1e-30) max(P_c[a][b],1e-30), EI = ED =
//                  sum_c w[g][c] max(pi_c[a],1e-30), wildcard factor 1.
//
// All arithmetic is float64; chi and the tables are rounded to float32 once,
// as the E-step consumes them.
#include "pairhmm.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <vector>

extern "C" __attribute__((visibility("hidden"))) void phmm_internal_set_error(const char *msg);

namespace pro {

constexpr int S = 0, M = 1, I = 2, D = 3, E = 4;
constexpr int NA = 20;                 // alphabet (residues 0..19)
constexpr int MAXV = 3960;             // doubles of the by-value parameter block
constexpr int MAXK = 33;               // K*F <= 33 keeps N <= 167
constexpr int THREADS = 256;

// Parameter block passed by value (kernel parameters hold up to 32 KB).
struct Packed {
    int K, F, C;
    int q_direct;   // 1: v + o_S holds the rate matrix Q itself (TKF models), 0: exchangeabilities S
    int o_dins, o_ddel, o_dw, o_fw, o_ext, o_pis, o_S, o_cd;
    double main_ins, main_del;
    double v[MAXV];
};

__device__ __constant__ int UV_U[5] = {M, M, M, I, D};
__device__ __constant__ int UV_X[5] = {M, I, D, I, D};
__device__ __constant__ int MID[3] = {M, I, D};

// ---------------------------------------------------------------- scalars
// The chi builder is written once for a scalar type T: double for the
// values, Dual (value and one directional derivative, forward mode) for the
// vector-Jacobian product of the gradient path.  Branches test values only
// and evaluate the selected expression alone, so a derivative is the
// derivative of the branch taken, as autograd through torch.where gives it.
struct Dual {
    double v, d;
};
__device__ __forceinline__ Dual mkd(double v, double d = 0.0) { return {v, d}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return {a - b.v, -b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, double b) { return {a.v / b, a.d / b}; }
__device__ __forceinline__ Dual operator/(double a, Dual b) {
    const double q = a / b.v;
    return {q, -q * b.d / b.v};
}
__device__ __forceinline__ Dual texp(Dual a) {
    const double e = exp(a.v);
    return {e, e * a.d};
}
__device__ __forceinline__ double texp(double a) { return exp(a); }
__device__ __forceinline__ double val(double a) { return a; }
__device__ __forceinline__ double val(Dual a) { return a.v; }
template <class T> __device__ __forceinline__ T cst(double c);
template <> __device__ __forceinline__ double cst<double>(double c) { return c; }
template <> __device__ __forceinline__ Dual cst<Dual>(double c) { return {c, 0.0}; }
// max(a, c) for a constant floor c (clamp_min): the floor has no derivative
template <class T> __device__ __forceinline__ T floor_at(T a, double c) { return val(a) > c ? a : cst<T>(c); }

// ---------------------------------------------------------------- TKF BDI (core/bdi.py:40-99)
template <class T>
__device__ T tkf_beta(T lam, T mu, T t) {
    const T s = mu * t;
    if (fabs(1.0 - val(lam) / val(mu)) < 1e-4) return s / (1.0 + s);
    const T eta = texp(-(lam * t));
    const T alpha = texp(-s);
    const T denom = mu * eta - lam * alpha;
    if (fabs(val(denom)) < 1e-30) return cst<T>(0.0);
    return lam * (eta - alpha) / denom;
}

template <class T>
__device__ T tkf_gamma(T lam, T mu, T t) {
    const T s = mu * t;
    const T alpha = texp(-(mu * t));
    const T Phi = 1.0 - alpha;
    if (fabs(1.0 - val(lam) / val(mu)) < 1e-4) {
        const T phi = val(s) < 1e-10 ? 1.0 - s / 2.0 : Phi / floor_at(s, 1e-30);
        return 1.0 - 1.0 / ((1.0 + s) * phi);
    }
    if (fabs(val(Phi)) < 1e-30) return cst<T>(0.0);
    const T beta = tkf_beta(lam, mu, t);
    return 1.0 - mu * beta / (lam * floor_at(Phi, 1e-30));
}

// [5][5] TKF91 pair-HMM matrix, order S, M, I, D, E (core/params.py:29-55)
template <class T>
__device__ void tkf91(T lam, T mu, T t, T *tau) {
    const T a = texp(-(mu * t)), b = tkf_beta(lam, mu, t), g = tkf_gamma(lam, mu, t);
    const T k = lam / mu;
    const T z = cst<T>(0.0);
    const T row[5] = {z, (1.0 - b) * k * a, b, (1.0 - b) * k * (1.0 - a), (1.0 - b) * (1.0 - k)};
    const T rowD[5] = {z, (1.0 - g) * k * a, g, (1.0 - g) * k * (1.0 - a), (1.0 - g) * (1.0 - k)};
    for (int v = 0; v < 5; ++v) {
        tau[S * 5 + v] = row[v];
        tau[M * 5 + v] = row[v];
        tau[I * 5 + v] = row[v];
        tau[D * 5 + v] = rowD[v];
        tau[E * 5 + v] = z;
    }
}

// ---------------------------------------------------------------- collapsed chi
// Shared layout of the chi builder (elements of T).
template <class T>
struct ChiSmem {
    int K, n3, w;             // K, 3K, 3K + 5 (row width of the solve matrix)
    T *tau, *tauK, *kap, *z, *Tex, *T5, *TnN, *ent, *exi, *aug;
    __device__ void carve(T *base, int K_) {
        K = K_;
        n3 = 3 * K_;
        w = n3 + 5;
        tau = base;                 // [25]
        tauK = tau + 25;            // [K][25]
        kap = tauK + 25 * K;        // [K]
        z = kap + K;                // [3K]     null probability of flat index 3k+e
        Tex = z + n3;               // [K][25]  T_exit_k
        T5 = Tex + 25 * K;          // [25]     effective T
        TnN = T5 + 25;              // [3K][5]  T_nullN
        ent = TnN + 5 * n3;         // [K][5]   entry factors
        exi = ent + 5 * K;          // [K][5]   exit factors (before notext)
        aug = exi + 5 * K;          // [3K][3K+5] solve matrix
    }
    __host__ __device__ static size_t elems(int K_) {
        const size_t n3 = 3 * (size_t)K_;
        return 25 + 25 * K_ + K_ + n3 + 25 * K_ + 25 + 5 * n3 + 10 * K_ + n3 * (n3 + 5);
    }
};

// The chi parameters seen by the builder: main rates, pair time and the
// packed domain arrays (dom_ins, dom_del, dom_w, frag_w, ext), as T.
template <class T>
struct ChiParams {
    T main_ins, main_del, t;
    const T *dins, *ddel, *dw, *fw, *ext;
};

// Build the N x N collapsed chi of one pair (models/mixdom.py:104-423) with
// the CTA; emit(idx, value) receives every entry (row-major, idx = r*N + c).
template <class T, class Emit>
__device__ void build_chi(const ChiParams<T> &cp, int K, int F, int N, ChiSmem<T> &sm, int *piv_row, Emit emit) {
    const int tid = threadIdx.x;
    const int n3 = sm.n3, w = sm.w;
    // TKF91 matrices of the main level and of each domain level
    if (tid == 0) tkf91(cp.main_ins, cp.main_del, cp.t, sm.tau);
    for (int k = tid; k < K; k += blockDim.x) {
        tkf91(cp.dins[k], cp.ddel[k], cp.t, sm.tauK + 25 * k);
        const T kap = cp.dins[k] / cp.ddel[k];
        const T zt = (1.0 - kap) * (1.0 - tkf_beta(cp.dins[k], cp.ddel[k], cp.t));
        sm.kap[k] = kap;
        sm.z[3 * k] = zt;
        sm.z[3 * k + 1] = 1.0 - kap;
        sm.z[3 * k + 2] = 1.0 - kap;
    }
    __syncthreads();

    // null-domain quantities (models/mixdom.py:104-214): for flat index
    // i = 3k + e (e over the M, I, D contexts), z(i) is the probability that
    // domain k emits nothing, T_nullN[i] its exits to the main level
    const T *tau = sm.tau;
    const T tauE[3] = {tau[M * 5 + E], tau[M * 5 + E], tau[D * 5 + E]};
    const int nullrow[3] = {M, M, D};
    for (int i = tid; i < n3; i += blockDim.x) {
        const int k = i / 3, e = i % 3;
        const T z = sm.z[i];
        const T nonnull = e == 0 ? 1.0 - z : sm.kap[k];
        for (int v = 0; v < 5; ++v) sm.TnN[i * 5 + v] = cst<T>(0.0);
        sm.TnN[i * 5 + MID[e]] = nonnull;
        sm.TnN[i * 5 + E] = z * tauE[e];
        // row i of the solve matrix is column i of (I - T_nn):
        // (I - T_nn)[j][i] = delta - z(j) dw[k(i)] tau[nullrow[e(j)]][MID[e(i)]]
        for (int j = 0; j < n3; ++j)
            sm.aug[i * w + j] = (i == j ? 1.0 : 0.0) - sm.z[j] * cp.dw[k] * tau[nullrow[j % 3] * 5 + MID[e]];
        // right-hand sides: T_Nnull[u][i] = tau[u][MID[e]] dw[k]
        for (int u = 0; u < 5; ++u) sm.aug[i * w + n3 + u] = tau[u * 5 + MID[e]] * cp.dw[k];
    }
    __syncthreads();

    // Gauss-Jordan with partial pivoting: (I - T_nn)^T Y^T = T_Nnull^T
    for (int c = 0; c < n3; ++c) {
        if (tid == 0) {
            int best = c;
            double bv = fabs(val(sm.aug[c * w + c]));
            for (int r = c + 1; r < n3; ++r) {
                const double v = fabs(val(sm.aug[r * w + c]));
                if (v > bv) { bv = v; best = r; }
            }
            *piv_row = best;
        }
        __syncthreads();
        const int pr = *piv_row;
        if (pr != c)
            for (int j = tid; j < w; j += blockDim.x) {
                const T a = sm.aug[c * w + j];
                sm.aug[c * w + j] = sm.aug[pr * w + j];
                sm.aug[pr * w + j] = a;
            }
        __syncthreads();
        const T inv = 1.0 / sm.aug[c * w + c];
        __syncthreads();
        for (int j = tid; j < w; j += blockDim.x) sm.aug[c * w + j] = sm.aug[c * w + j] * inv;
        __syncthreads();
        for (int idx = tid; idx < n3 * w; idx += blockDim.x) {
            const int r = idx / w, j = idx % w;
            if (r == c || j == c) continue;
            sm.aug[idx] = sm.aug[idx] - sm.aug[r * w + c] * sm.aug[c * w + j];
        }
        __syncthreads();
        for (int r = tid; r < n3; r += blockDim.x)
            if (r != c) sm.aug[r * w + c] = cst<T>(0.0);
        __syncthreads();
    }

    // T_exit_k[k][u][v] = sum_e Y[u][3k+e] T_nullN[3k+e][v]; Y[u][i] = aug[i][3K+u]
    for (int idx = tid; idx < 25 * K; idx += blockDim.x) {
        const int k = idx / 25, u = (idx / 5) % 5, v = idx % 5;
        T s = cst<T>(0.0);
        for (int e = 0; e < 3; ++e) s = s + sm.aug[(3 * k + e) * w + n3 + u] * sm.TnN[(3 * k + e) * 5 + v];
        sm.Tex[idx] = s;
    }
    // entry / exit factors of each domain's five sub-states
    for (int idx = tid; idx < 5 * K; idx += blockDim.x) {
        const int k = idx / 5, j = idx % 5;
        const T *tk = sm.tauK + 25 * k;
        const T beta_d = floor_at(1.0 - tk[S * 5 + E], 1e-30);
        const bool isM = j < 3;
        sm.ent[idx] = isM ? tk[S * 5 + UV_X[j]] / beta_d : cst<T>(1.0);
        sm.exi[idx] = isM ? tk[UV_X[j] * 5 + E] : 1.0 - sm.kap[k];
    }
    __syncthreads();
    for (int idx = tid; idx < 25; idx += blockDim.x) {
        T s = (idx % 5 == E) ? tau[idx] : cst<T>(0.0);
        for (int k = 0; k < K; ++k) s = s + sm.Tex[25 * k + idx];
        sm.T5[idx] = s;
    }
    __syncthreads();

    // chi (models/mixdom.py:252-423): state 0 = SS, 1 = EE, body state
    // 2 + k*5F + j*F + f (domain k, sub-state j, fragment f)
    const int bs = 5 * F;
    for (int idx = tid; idx < N * N; idx += blockDim.x) {
        const int r = idx / N, c = idx % N;
        T v = cst<T>(0.0);
        if (r == 0) {
            if (c == 1) {
                v = sm.T5[S * 5 + E];
            } else if (c >= 2) {
                const int q = c - 2, kq = q / bs, jq = (q % bs) / F, fq = q % F;
                v = sm.Tex[25 * kq + S * 5 + UV_U[jq]] * cp.fw[kq * F + fq] * sm.ent[5 * kq + jq];
            }
        } else if (r >= 2 && c >= 1) {
            const int pp = r - 2, kp = pp / bs, jp = (pp % bs) / F, fp = pp % F;
            T notext = cst<T>(1.0);
            for (int g = 0; g < F; ++g) notext = notext - cp.ext[(kp * F + fp) * F + g];
            const T exit_full = notext * sm.exi[5 * kp + jp];
            if (c == 1) {
                v = exit_full * sm.T5[UV_U[jp] * 5 + E];
            } else {
                const int q = c - 2, kq = q / bs, jq = (q % bs) / F, fq = q % F;
                const T dest = cp.fw[kq * F + fq] * sm.ent[5 * kq + jq];
                v = exit_full * sm.Tex[25 * kq + UV_U[jp] * 5 + UV_U[jq]] * dest;
                if (kp == kq) {
                    const T e = cp.ext[(kp * F + fp) * F + fq];
                    if (jp < 3 && jq < 3)
                        v = v + notext * sm.tauK[25 * kp + MID[jp] * 5 + MID[jq]] * cp.fw[kp * F + fq] +
                            (jp == jq ? e : cst<T>(0.0));
                    else if (jp == jq)
                        v = v + notext * sm.kap[kp] * cp.fw[kp * F + fq] + e;
                }
            }
        }
        emit(idx, v);
    }
}

// The factored form of chi (models/mixdom.py:343-394) from the builder's
// intermediate results (after build_chi): per body state q = d*5F + j*F + f,
// exit[q] = notext[d,f] exi[d,j]; cin[a][q] = T_exit_k[d][a][U(j)] dest[q]
// for the top-level types a = M, I, D; and each domain's same-domain block
// without its inter part, intra[d][j'F+f'][jF+f] (the M-block couples the
// sub-states MM, MI, MD; II and DD couple within themselves).  Layout of
// phmm_batch.nest: exit [nb], cin [3][nb], intra [K][5F][5F].
template <class T>
__device__ void write_nest(const ChiParams<T> &cp, int K, int F, const ChiSmem<T> &sm, float *rec) {
    const int nb = 5 * K * F, bs = 5 * F;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        const int k = q / bs, j = (q % bs) / F, f = q % F;
        T notext = cst<T>(1.0);
        for (int g = 0; g < F; ++g) notext = notext - cp.ext[(k * F + f) * F + g];
        rec[q] = (float)(notext * sm.exi[5 * k + j]);
        const T dest = cp.fw[k * F + f] * sm.ent[5 * k + j];
        for (int a = 0; a < 3; ++a) rec[nb + a * nb + q] = (float)(sm.Tex[25 * k + MID[a] * 5 + UV_U[j]] * dest);
    }
    for (int idx = threadIdx.x; idx < K * bs * bs; idx += blockDim.x) {
        const int k = idx / (bs * bs), i = (idx / bs) % bs, c = idx % bs;
        const int jp = i / F, fp = i % F, jq = c / F, fq = c % F;
        T v = cst<T>(0.0);
        if ((jp < 3 && jq < 3) || jp == jq) {
            T notext = cst<T>(1.0);
            for (int g = 0; g < F; ++g) notext = notext - cp.ext[(k * F + fp) * F + g];
            const T e = cp.ext[(k * F + fp) * F + fq];
            if (jp < 3 && jq < 3)
                v = notext * sm.tauK[25 * k + MID[jp] * 5 + MID[jq]] * cp.fw[k * F + fq] + (jp == jq ? e : cst<T>(0.0));
            else
                v = notext * sm.kap[k] * cp.fw[k * F + fq] + e;
        }
        rec[4 * nb + idx] = (float)v;
    }
}

// chi (nullable), its float64 copy (nullable) and the factored record (nullable) of pair blockIdx.x
__device__ __forceinline__ void chi_kernel_body(const Packed &prm, const double *__restrict__ ts, int N, float *__restrict__ chi,
           double *__restrict__ chi64, float *__restrict__ nest = nullptr) {
    extern __shared__ double smem_d[];
    __shared__ int piv_row;
    const int p = blockIdx.x;
    ChiSmem<double> sm;
    sm.carve(smem_d, prm.K);
    const ChiParams<double> cp{prm.main_ins, prm.main_del, ts[p], prm.v + prm.o_dins, prm.v + prm.o_ddel,
                               prm.v + prm.o_dw, prm.v + prm.o_fw, prm.v + prm.o_ext};
    float *out = chi ? chi + (size_t)p * N * N : nullptr;
    double *out64 = chi64 ? chi64 + (size_t)p * N * N : nullptr;
    build_chi(cp, prm.K, prm.F, N, sm, &piv_row, [&](int idx, double v) {
        if (out) out[idx] = (float)v;
        if (out64) out64[idx] = v;
    });
    if (nest) {
        __syncthreads();
        const int K = prm.K, F = prm.F;
        write_nest(cp, K, F, sm, nest + (size_t)p * (20 * K * F + 25 * K * F * F));
    }
}

__global__ void __launch_bounds__(THREADS)
nest_kernel(const __grid_constant__ Packed prm, const double *__restrict__ ts, int N, float *__restrict__ nest) {
    chi_kernel_body(prm, ts, N, nullptr, nullptr, nest);
}

__global__ void __launch_bounds__(THREADS)
nest_kernel_dp(const Packed *__restrict__ prm, const double *__restrict__ ts, int N, float *__restrict__ nest) {
    chi_kernel_body(*prm, ts, N, nullptr, nullptr, nest);
}

__global__ void __launch_bounds__(THREADS)
chi_kernel(const __grid_constant__ Packed prm, const double *__restrict__ ts, int N, float *__restrict__ chi, double *__restrict__ chi64,
           float *__restrict__ nest = nullptr) {
    chi_kernel_body(prm, ts, N, chi, chi64, nest);
}

// the same with the parameter block in device memory (a captured graph
// refreshes it by a copy before each replay)
__global__ void __launch_bounds__(THREADS)
chi_kernel_dp(const Packed *__restrict__ prm, const double *__restrict__ ts, int N, float *__restrict__ chi, double *__restrict__ chi64,
              float *__restrict__ nest = nullptr) {
    chi_kernel_body(*prm, ts, N, chi, chi64, nest);
}

// Vector-Jacobian product of chi: for pair p = blockIdx.x and parameter
// direction d = blockIdx.y, grad[p][d] = sum_{s,k} G[p][s][k] dchi[s][k]/dtheta_d,
// by one forward-mode (Dual) pass of the builder seeded on theta_d.
// Directions: 0 main_ins, 1 main_del, 2 t, 3 + j the j-th entry of the packed
// domain arrays (dom_ins[K], dom_del[K], dom_w[K], frag_w[K*F], ext[K*F*F]).
__global__ void __launch_bounds__(THREADS)
chi_vjp_kernel(const __grid_constant__ Packed prm, const double *__restrict__ ts, int N,
               const double *__restrict__ G, double *__restrict__ grad) {
    extern __shared__ Dual smem_dual[];
    __shared__ int piv_row;
    __shared__ double red[THREADS / 32];
    const int p = blockIdx.x, dir = blockIdx.y, nd = gridDim.y, tid = threadIdx.x;
    const int K = prm.K, F = prm.F;
    const int nparam = 3 * K + K * F + K * F * F;
    ChiSmem<Dual> sm;
    sm.carve(smem_dual, K);
    Dual *pv = smem_dual + ChiSmem<Dual>::elems(K);   // the packed domain arrays as Duals
    for (int j = tid; j < nparam; j += blockDim.x) pv[j] = mkd(prm.v[prm.o_dins + j], dir == 3 + j ? 1.0 : 0.0);
    __syncthreads();
    const ChiParams<Dual> cp{mkd(prm.main_ins, dir == 0 ? 1.0 : 0.0), mkd(prm.main_del, dir == 1 ? 1.0 : 0.0),
                             mkd(ts[p], dir == 2 ? 1.0 : 0.0), pv, pv + K, pv + 2 * K, pv + 3 * K,
                             pv + 3 * K + K * F};
    const double *Gp = G + (size_t)p * N * N;
    double acc = 0.0;
    build_chi(cp, K, F, N, sm, &piv_row, [&](int idx, Dual v) { acc += Gp[idx] * v.d; });
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
    __syncthreads();
    if (tid == 0) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
        grad[(size_t)p * nd + dir] = s;
    }
}

// ---------------------------------------------------------------- expm (Pade 13)
// b_j of the [13/13] Pade approximant of exp (Higham 2005, eq. 2.1 / Table 2.3)
__device__ __constant__ double PADE13[14] = {
    64764752532480000.0, 32382376266240000.0, 7771770303897600.0, 1187353796428800.0,
    129060195264000.0, 10559470521600.0, 670442572800.0, 33522128640.0,
    1323241920.0, 40840800.0, 960960.0, 16380.0, 182.0, 1.0};
// theta_13 of the same paper: the 1-norm up to which degree 13 needs no scaling
constexpr double THETA13 = 5.371920351148152;

__device__ void mm(double *C, const double *A, const double *B, int n) {
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        const int i = idx / n, j = idx % n;
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += A[i * n + k] * B[k * n + j];
        C[idx] = s;
    }
    __syncthreads();
}

__device__ __forceinline__ void expm_kernel_body(const Packed &prm, const double *__restrict__ ts, double *__restrict__ csubs) {
    constexpr int n = NA, nn = NA * NA;
    __shared__ double X[nn], A2[nn], A4[nn], A6[nn], W1[nn], W2[nn], U[nn], V[nn];
    __shared__ double aug[n * 2 * n];
    __shared__ double colsum[n];
    __shared__ int piv_row, n_sq;
    const int p = blockIdx.x / prm.C, c = blockIdx.x % prm.C, tid = threadIdx.x;
    const double t = ts[p];
    const double *Sx = prm.v + prm.o_S + (size_t)c * nn, *pi = prm.v + prm.o_pis + c * n;

    if (prm.q_direct) {   // the caller's rate matrix (core/ctmc.py:31-60 takes Q as given)
        for (int idx = tid; idx < nn; idx += blockDim.x) X[idx] = Sx[idx];
    } else {
        // Q[a][b] = S[a][b] pi[b] off the diagonal, rows summing to zero (train/vjp.py:463-476)
        for (int idx = tid; idx < nn; idx += blockDim.x) {
            const int a = idx / n, b = idx % n;
            X[idx] = a == b ? 0.0 : Sx[idx] * pi[b];
        }
        __syncthreads();
        if (tid < n) {
            double s = 0.0;
            for (int b = 0; b < n; ++b) s += X[tid * n + b];
            X[tid * n + tid] = -s;
        }
    }
    __syncthreads();
    for (int idx = tid; idx < nn; idx += blockDim.x) X[idx] *= t;
    __syncthreads();
    if (tid < n) {
        double s = 0.0;
        for (int a = 0; a < n; ++a) s += fabs(X[a * n + tid]);
        colsum[tid] = s;
    }
    __syncthreads();
    if (tid == 0) {
        double nrm = 0.0;
        for (int b = 0; b < n; ++b) nrm = fmax(nrm, colsum[b]);
        int s = 0;
        if (nrm > THETA13) s = (int)ceil(log2(nrm / THETA13));
        n_sq = s < 0 ? 0 : (s > 60 ? 60 : s);
    }
    __syncthreads();
    const int s = n_sq;
    for (int idx = tid; idx < nn; idx += blockDim.x) X[idx] = ldexp(X[idx], -s);
    __syncthreads();
    mm(A2, X, X, n);
    mm(A4, A2, A2, n);
    mm(A6, A4, A2, n);
    const double *b = PADE13;
    // W1 = b13 A6 + b11 A4 + b9 A2;  W2 = b12 A6 + b10 A4 + b8 A2
    for (int idx = tid; idx < nn; idx += blockDim.x) {
        W1[idx] = b[13] * A6[idx] + b[11] * A4[idx] + b[9] * A2[idx];
        W2[idx] = b[12] * A6[idx] + b[10] * A4[idx] + b[8] * A2[idx];
    }
    __syncthreads();
    mm(U, A6, W1, n);   // A6 W1
    mm(V, A6, W2, n);   // A6 W2
    for (int idx = tid; idx < nn; idx += blockDim.x) {
        const double id = (idx / n == idx % n) ? 1.0 : 0.0;
        W1[idx] = U[idx] + b[7] * A6[idx] + b[5] * A4[idx] + b[3] * A2[idx] + b[1] * id;
        V[idx] = V[idx] + b[6] * A6[idx] + b[4] * A4[idx] + b[2] * A2[idx] + b[0] * id;
    }
    __syncthreads();
    mm(U, X, W1, n);    // U = X (A6 W1 + ...)
    // solve (V - U) R = (V + U)
    for (int idx = tid; idx < nn; idx += blockDim.x) {
        const int i = idx / n, j = idx % n;
        aug[i * 2 * n + j] = V[idx] - U[idx];
        aug[i * 2 * n + n + j] = V[idx] + U[idx];
    }
    __syncthreads();
    const int w = 2 * n;
    for (int cc = 0; cc < n; ++cc) {
        if (tid == 0) {
            int best = cc;
            double bv = fabs(aug[cc * w + cc]);
            for (int r = cc + 1; r < n; ++r) {
                const double v = fabs(aug[r * w + cc]);
                if (v > bv) { bv = v; best = r; }
            }
            piv_row = best;
        }
        __syncthreads();
        const int pr = piv_row;
        if (pr != cc)
            for (int j = tid; j < w; j += blockDim.x) {
                const double a = aug[cc * w + j];
                aug[cc * w + j] = aug[pr * w + j];
                aug[pr * w + j] = a;
            }
        __syncthreads();
        const double inv = 1.0 / aug[cc * w + cc];
        __syncthreads();
        for (int j = tid; j < w; j += blockDim.x) aug[cc * w + j] *= inv;
        __syncthreads();
        for (int idx = tid; idx < n * w; idx += blockDim.x) {
            const int r = idx / w, j = idx % w;
            if (r == cc || j == cc) continue;
            aug[idx] -= aug[r * w + cc] * aug[cc * w + j];
        }
        __syncthreads();
        for (int r = tid; r < n; r += blockDim.x)
            if (r != cc) aug[r * w + cc] = 0.0;
        __syncthreads();
    }
    for (int idx = tid; idx < nn; idx += blockDim.x) W1[idx] = aug[(idx / n) * w + n + idx % n];
    __syncthreads();
    // undo the scaling: square s times
    double *cur = W1, *nxt = W2;
    for (int k = 0; k < s; ++k) {
        mm(nxt, cur, cur, n);
        double *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    double *out = csubs + ((size_t)p * prm.C + c) * nn;
    for (int idx = tid; idx < nn; idx += blockDim.x) out[idx] = cur[idx];
}

__global__ void __launch_bounds__(THREADS)
expm_kernel(const __grid_constant__ Packed prm, const double *__restrict__ ts, double *__restrict__ csubs) {
    expm_kernel_body(prm, ts, csubs);
}

// the same with the parameter block in device memory (a captured graph
// refreshes it by a copy before each replay)
__global__ void __launch_bounds__(THREADS)
expm_kernel_dp(const Packed *__restrict__ prm, const double *__restrict__ ts, double *__restrict__ csubs) {
    expm_kernel_body(*prm, ts, csubs);
}

// ---------------------------------------------------------------- emission tables
__device__ __forceinline__ void tables_kernel_body(const Packed &prm, const double *__restrict__ csubs, float *__restrict__ EM,
              float *__restrict__ EI, float *__restrict__ ED) {
    const int p = blockIdx.x, tid = threadIdx.x;
    const int C = prm.C, G = prm.K * prm.F;
    const double *cd = prm.v + prm.o_cd, *pis = prm.v + prm.o_pis;
    const double *Pp = csubs + (size_t)p * C * NA * NA;
    float *em = EM + (size_t)p * G * 441;
    for (int idx = tid; idx < G * 441; idx += blockDim.x) {
        const int g = idx / 441, a = (idx / 21) % 21, bb = idx % 21;
        double s = 0.0;
        for (int c = 0; c < C; ++c) {
            const double lp = a < NA ? fmax(pis[c * NA + a], 1e-30) : 1.0;
            const double ls = (a < NA && bb < NA) ? fmax(Pp[(c * NA + a) * NA + bb], 1e-30) : 1.0;
            s += cd[g * C + c] * (lp * ls);
        }
        em[idx] = (float)s;
    }
    for (int idx = tid; idx < G * 21; idx += blockDim.x) {
        const int g = idx / 21, a = idx % 21;
        double s = 0.0;
        for (int c = 0; c < C; ++c) s += cd[g * C + c] * (a < NA ? fmax(pis[c * NA + a], 1e-30) : 1.0);
        EI[(size_t)p * G * 21 + idx] = (float)s;
        ED[(size_t)p * G * 21 + idx] = (float)s;
    }
}

__global__ void __launch_bounds__(THREADS)
tables_kernel(const __grid_constant__ Packed prm, const double *__restrict__ csubs, float *__restrict__ EM, float *__restrict__ EI, float *__restrict__ ED) {
    tables_kernel_body(prm, csubs, EM, EI, ED);
}

// the same with the parameter block in device memory (a captured graph
// refreshes it by a copy before each replay)
__global__ void __launch_bounds__(THREADS)
tables_kernel_dp(const Packed *__restrict__ prm, const double *__restrict__ csubs, float *__restrict__ EM, float *__restrict__ EI, float *__restrict__ ED) {
    tables_kernel_body(*prm, csubs, EM, EI, ED);
}

// ---------------------------------------------------------------- class split (epilogue)
// Per-class counts of train/likelihood.py:279-344 from the per-(d,f) character
// tables: the class posterior of a cell depends on it only through its
// characters, so with f_c[a][b] = pi_c[a'] P_c[a'][b'] (a' = min(a, A-1):
// the reference's clamped gather for the wildcard) and w[g][c] = classdist,
//   match[c][a][b] = sum_g cM[g][a][b] w[g][c] f_c[a][b] / sum_c' w[g][c'] f_c'[a][b]
// (insert / delete alike with pi_c[a']), classdist[g][c] = the sum over all
// 21 x 21 (and 21) characters of the same terms.  One CTA per pair.
constexpr int CS_MAXC = 8;

__device__ __forceinline__ void class_split_kernel_body(const Packed &prm, const double *__restrict__ csubs,
                   const double *__restrict__ cM, const double *__restrict__ cI, const double *__restrict__ cD,
                   double *__restrict__ match, double *__restrict__ ins, double *__restrict__ del,
                   double *__restrict__ cdist) {
    extern __shared__ double cs_acc[];   // [G][C] classdist partial sums
    const int p = blockIdx.x, tid = threadIdx.x;
    const int C = prm.C, G = prm.K * prm.F;
    const double *cd = prm.v + prm.o_cd, *pis = prm.v + prm.o_pis;
    const double *Pp = csubs + (size_t)p * C * NA * NA;
    for (int i = tid; i < G * C; i += blockDim.x) cs_acc[i] = 0.0;
    __syncthreads();
    double loc[CS_MAXC];
    // match-type cells
    for (int ab = tid; ab < 441; ab += blockDim.x) {
        const int a = ab / 21, b = ab % 21;
        const int ac = a < NA ? a : NA - 1, bc = b < NA ? b : NA - 1;
        double f[CS_MAXC], acc[CS_MAXC];
        for (int c = 0; c < C; ++c) {
            f[c] = pis[c * NA + ac] * Pp[(c * NA + ac) * NA + bc];
            acc[c] = 0.0;
        }
        for (int g = 0; g < G; ++g) {
            double den = 0.0;
            for (int c = 0; c < C; ++c) den += cd[g * C + c] * f[c];
            const double n = cM[((size_t)p * G + g) * 441 + ab];
            for (int c = 0; c < C; ++c) {
                const double wgc = n * (cd[g * C + c] * f[c] / (den + 1e-300));
                acc[c] += wgc;
                loc[c] = wgc;
            }
            for (int c = 0; c < C; ++c) atomicAdd(&cs_acc[g * C + c], loc[c]);
        }
        if (a < NA && b < NA)
            for (int c = 0; c < C; ++c) match[(((size_t)p * C + c) * NA + a) * NA + b] = acc[c];
    }
    // insert / delete cells: the same posterior over pi_c
    for (int ia = tid; ia < 2 * 21; ia += blockDim.x) {
        const bool is_ins = ia < 21;
        const int a = ia % 21, ac = a < NA ? a : NA - 1;
        const double *cnt = is_ins ? cI : cD;
        double acc[CS_MAXC];
        for (int c = 0; c < C; ++c) acc[c] = 0.0;
        for (int g = 0; g < G; ++g) {
            double den = 0.0;
            for (int c = 0; c < C; ++c) den += cd[g * C + c] * pis[c * NA + ac];
            const double n = cnt[((size_t)p * G + g) * 21 + a];
            for (int c = 0; c < C; ++c) {
                const double wgc = n * (cd[g * C + c] * pis[c * NA + ac] / (den + 1e-300));
                acc[c] += wgc;
                atomicAdd(&cs_acc[g * C + c], wgc);
            }
        }
        if (a < NA) {
            double *out = is_ins ? ins : del;
            for (int c = 0; c < C; ++c) out[((size_t)p * C + c) * NA + a] = acc[c];
        }
    }
    __syncthreads();
    for (int i = tid; i < G * C; i += blockDim.x) cdist[(size_t)p * G * C + i] = cs_acc[i];
}

__global__ void __launch_bounds__(THREADS)
class_split_kernel(const __grid_constant__ Packed prm, const double *__restrict__ csubs, const double *__restrict__ cM, const double *__restrict__ cI, const double *__restrict__ cD, double *__restrict__ match, double *__restrict__ ins, double *__restrict__ del, double *__restrict__ cdist) {
    class_split_kernel_body(prm, csubs, cM, cI, cD, match, ins, del, cdist);
}

// the same with the parameter block in device memory (a captured graph
// refreshes it by a copy before each replay)
__global__ void __launch_bounds__(THREADS)
class_split_kernel_dp(const Packed *__restrict__ prm, const double *__restrict__ csubs, const double *__restrict__ cM, const double *__restrict__ cI, const double *__restrict__ cD, double *__restrict__ match, double *__restrict__ ins, double *__restrict__ del, double *__restrict__ cdist) {
    class_split_kernel_body(*prm, csubs, cM, cI, cD, match, ins, del, cdist);
}

// ---------------------------------------------------------------- TKF92 prologue
// chi = TKF92 [5][5] (core/params.py:94-133: M/I/D rows scaled by 1 - ext,
// ext added on their diagonal) with every entry floored at 1e-30, the
// log(max(tau, 1e-30)) of train/tkf92_svi_bw.py:164; one thread per pair.
__global__ void tkf92_chi_kernel(double lam, double mu, double ext, const double *__restrict__ ts, int P,
                                 float *__restrict__ chi) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    double tau[25];
    tkf91(lam, mu, ts[p], tau);
    for (int u = 0; u < 5; ++u)
        for (int v = 0; v < 5; ++v) {
            const bool emit_row = u == M || u == I || u == D;
            double x = emit_row ? tau[u * 5 + v] * (1.0 - ext) + (u == v ? ext : 0.0) : tau[u * 5 + v];
            chi[(size_t)p * 25 + u * 5 + v] = (float)fmax(x, 1e-30);
        }
}

// pair-HMM emission tables of one substitution model (dp/hmm.py:628-670):
// EM[a][b] = (pi[a] + 1e-30)(P[a][b] + 1e-30), EI = ED = pi + 1e-30, wildcard 1
struct TkfPi { double v[NA]; };

__global__ void __launch_bounds__(THREADS)
tkf_tables_kernel_v(const TkfPi pi, const double *__restrict__ sub, float *__restrict__ EM,
                    float *__restrict__ EI, float *__restrict__ ED) {
    const int p = blockIdx.x, tid = threadIdx.x;
    const double *Pp = sub + (size_t)p * NA * NA;
    for (int idx = tid; idx < 441; idx += blockDim.x) {
        const int a = idx / 21, b = idx % 21;
        const double lp = a < NA ? pi.v[a] + 1e-30 : 1.0;
        const double ls = (a < NA && b < NA) ? Pp[a * NA + b] + 1e-30 : 1.0;
        EM[(size_t)p * 441 + idx] = (float)(lp * ls);
    }
    for (int a = tid; a < 21; a += blockDim.x) {
        const float v = (float)(a < NA ? pi.v[a] + 1e-30 : 1.0);
        EI[(size_t)p * 21 + a] = v;
        ED[(size_t)p * 21 + a] = v;
    }
}

}  // namespace pro

static int pro_fail(int code, const char *msg) {
    phmm_internal_set_error(msg);
    return code;
}

static int pack_params(const phmm_mixdom2_params *prm, pro::Packed &pk, const char *who) {
    using namespace pro;
    char msg[160];
    if (!prm) {
        snprintf(msg, sizeof msg, "%s: null parameters", who);
        return pro_fail(PHMM_E_ARG, msg);
    }
    const int K = prm->n_dom, F = prm->n_frag, C = prm->n_classes;
    if (K < 1 || F < 1 || C < 1 || K * F > MAXK) {
        snprintf(msg, sizeof msg, "%s: need n_dom, n_frag, n_classes >= 1 and n_dom*n_frag <= 33", who);
        return pro_fail(PHMM_E_ARG, msg);
    }
    if (prm->alphabet != NA) {
        snprintf(msg, sizeof msg, "%s: alphabet must be 20", who);
        return pro_fail(PHMM_E_ARG, msg);
    }
    if (!prm->dom_ins || !prm->dom_del || !prm->dom_weights || !prm->frag_weights || !prm->ext_rates ||
        !prm->class_pis || !prm->class_S_exch || !prm->classdist) {
        snprintf(msg, sizeof msg, "%s: null host parameter array", who);
        return pro_fail(PHMM_E_ARG, msg);
    }
    const int need = 3 * K + K * F + K * F * F + C * NA + C * NA * NA + K * F * C;
    if (need > MAXV) {
        snprintf(msg, sizeof msg, "%s: parameter block too large (reduce n_classes)", who);
        return pro_fail(PHMM_E_ARG, msg);
    }
    std::memset(&pk, 0, sizeof(pk));
    pk.K = K;
    pk.F = F;
    pk.C = C;
    pk.main_ins = prm->main_ins;
    pk.main_del = prm->main_del;
    int o = 0;
    auto put = [&](const double *src, int count) {
        const int at = o;
        std::memcpy(pk.v + o, src, sizeof(double) * count);
        o += count;
        return at;
    };
    pk.o_dins = put(prm->dom_ins, K);
    pk.o_ddel = put(prm->dom_del, K);
    pk.o_dw = put(prm->dom_weights, K);
    pk.o_fw = put(prm->frag_weights, K * F);
    pk.o_ext = put(prm->ext_rates, K * F * F);
    pk.o_pis = put(prm->class_pis, C * NA);
    pk.o_S = put(prm->class_S_exch, C * NA * NA);
    pk.o_cd = put(prm->classdist, K * F * C);
    return PHMM_OK;
}

extern "C" size_t phmm_mixdom2_class_subs_count(const phmm_mixdom2_params *prm, int32_t n_pairs) {
    if (!prm || n_pairs < 0) return 0;
    return (size_t)n_pairs * prm->n_classes * pro::NA * pro::NA;
}

static int mixdom2_tables(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t, float *chi,
                          float *emit_M, float *emit_I, float *emit_D, double *class_subs, float *nest, void *stream);

extern "C" int phmm_mixdom2_tables(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t, float *chi,
                                   float *emit_M, float *emit_I, float *emit_D, double *class_subs, void *stream) {
    return mixdom2_tables(prm, n_pairs, t, chi, emit_M, emit_I, emit_D, class_subs, nullptr, stream);
}

extern "C" int phmm_mixdom2_tables_nest(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t, float *chi,
                                        float *emit_M, float *emit_I, float *emit_D, double *class_subs, float *nest,
                                        void *stream) {
    if (!nest && n_pairs > 0) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_tables_nest: null nest buffer");
    return mixdom2_tables(prm, n_pairs, t, chi, emit_M, emit_I, emit_D, class_subs, nest, stream);
}

static int mixdom2_tables(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t, float *chi,
                          float *emit_M, float *emit_I, float *emit_D, double *class_subs, float *nest, void *stream) {
    using namespace pro;
    Packed pk;
    int rc = pack_params(prm, pk, "phmm_mixdom2_tables");
    if (rc) return rc;
    if (n_pairs < 0) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_tables: negative n_pairs");
    if (n_pairs == 0) return PHMM_OK;
    if (!t || !chi || !emit_M || !emit_I || !emit_D || !class_subs)
        return pro_fail(PHMM_E_ARG, "phmm_mixdom2_tables: null device buffer");
    const int K = pk.K, F = pk.F, C = pk.C;
    const int N = 2 + 5 * K * F;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t chi_smem = sizeof(double) * ChiSmem<double>::elems(K);
    if (chi_smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(chi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)chi_smem);
        if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    }
    chi_kernel<<<n_pairs, THREADS, chi_smem, st>>>(pk, t, N, chi, nullptr, nest);
    expm_kernel<<<n_pairs * C, THREADS, 0, st>>>(pk, t, class_subs);
    tables_kernel<<<n_pairs, THREADS, 0, st>>>(pk, class_subs, emit_M, emit_I, emit_D);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

extern "C" int phmm_mixdom2_class_counts(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *class_subs,
                                         const double *cnt_M, const double *cnt_I, const double *cnt_D,
                                         double *class_match, double *class_insert, double *class_delete,
                                         double *classdist_counts, void *stream) {
    using namespace pro;
    Packed pk;
    int rc = pack_params(prm, pk, "phmm_mixdom2_class_counts");
    if (rc) return rc;
    if (pk.C > CS_MAXC) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_class_counts: at most 8 classes");
    if (n_pairs < 0) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_class_counts: negative n_pairs");
    if (n_pairs == 0) return PHMM_OK;
    if (!class_subs || !cnt_M || !cnt_I || !cnt_D || !class_match || !class_insert || !class_delete ||
        !classdist_counts)
        return pro_fail(PHMM_E_ARG, "phmm_mixdom2_class_counts: null device buffer");
    const size_t smem = sizeof(double) * pk.K * pk.F * pk.C;
    class_split_kernel<<<n_pairs, THREADS, smem, (cudaStream_t)stream>>>(
        pk, class_subs, cnt_M, cnt_I, cnt_D, class_match, class_insert, class_delete, classdist_counts);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

extern "C" int phmm_tkf92_tables(const phmm_tkf92_params *prm, int32_t n_pairs, const double *t, float *chi,
                                 float *emit_M, float *emit_I, float *emit_D, double *sub, void *stream) {
    using namespace pro;
    if (!prm) return pro_fail(PHMM_E_ARG, "phmm_tkf92_tables: null parameters");
    if (prm->alphabet != NA) return pro_fail(PHMM_E_ARG, "phmm_tkf92_tables: alphabet must be 20");
    if (!prm->Q || !prm->pi) return pro_fail(PHMM_E_ARG, "phmm_tkf92_tables: null host parameter array");
    if (!(prm->ins_rate > 0.0) || !(prm->del_rate > 0.0) || !(prm->ext >= 0.0 && prm->ext < 1.0))
        return pro_fail(PHMM_E_ARG, "phmm_tkf92_tables: need ins_rate, del_rate > 0 and 0 <= ext < 1");
    if (n_pairs < 0) return pro_fail(PHMM_E_ARG, "phmm_tkf92_tables: negative n_pairs");
    if (n_pairs == 0) return PHMM_OK;
    if (!t || !chi || !emit_M || !emit_I || !emit_D || !sub)
        return pro_fail(PHMM_E_ARG, "phmm_tkf92_tables: null device buffer");
    Packed pk;
    std::memset(&pk, 0, sizeof(pk));
    pk.C = 1;
    pk.q_direct = 1;
    pk.o_S = 0;
    std::memcpy(pk.v, prm->Q, sizeof(double) * NA * NA);
    TkfPi pv;
    std::memcpy(pv.v, prm->pi, sizeof(double) * NA);
    cudaStream_t st = (cudaStream_t)stream;
    tkf92_chi_kernel<<<(n_pairs + 127) / 128, 128, 0, st>>>(prm->ins_rate, prm->del_rate, prm->ext, t, n_pairs, chi);
    expm_kernel<<<n_pairs, THREADS, 0, st>>>(pk, t, sub);
    tkf_tables_kernel_v<<<n_pairs, THREADS, 0, st>>>(pv, sub, emit_M, emit_I, emit_D);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

extern "C" int phmm_mixdom2_chi(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t, float *chi,
                                double *chi64, void *stream) {
    using namespace pro;
    Packed pk;
    int rc = pack_params(prm, pk, "phmm_mixdom2_chi");
    if (rc) return rc;
    if (n_pairs < 0) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_chi: negative n_pairs");
    if (n_pairs == 0) return PHMM_OK;
    if (!t || !chi) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_chi: null device buffer");
    const int N = 2 + 5 * pk.K * pk.F;
    const size_t smem = sizeof(double) * ChiSmem<double>::elems(pk.K);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(chi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    }
    chi_kernel<<<n_pairs, THREADS, smem, (cudaStream_t)stream>>>(pk, t, N, chi, chi64);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

extern "C" int phmm_mixdom2_chi_vjp_dirs(const phmm_mixdom2_params *prm) {
    if (!prm) return 0;
    const int K = prm->n_dom, F = prm->n_frag;
    return 3 + 3 * K + K * F + K * F * F;
}

extern "C" int phmm_mixdom2_chi_vjp(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t,
                                    const double *grad_chi, double *grad, void *stream) {
    using namespace pro;
    Packed pk;
    int rc = pack_params(prm, pk, "phmm_mixdom2_chi_vjp");
    if (rc) return rc;
    if (n_pairs < 0) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_chi_vjp: negative n_pairs");
    if (n_pairs == 0) return PHMM_OK;
    if (!t || !grad_chi || !grad) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_chi_vjp: null device buffer");
    const int K = pk.K, F = pk.F;
    const int N = 2 + 5 * K * F;
    const int nd = 3 + 3 * K + K * F + K * F * F;
    const size_t smem = sizeof(Dual) * (ChiSmem<Dual>::elems(K) + (size_t)(nd - 3));
    if (smem > 227 * 1024) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_chi_vjp: state space too large");
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(chi_vjp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    }
    chi_vjp_kernel<<<dim3(n_pairs, nd), THREADS, smem, (cudaStream_t)stream>>>(pk, t, N, grad_chi, grad);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

// ---------------------------------------------------------------- Holmes-Rubin statistics
// Per (pair, class) endpoint-conditioned substitution statistics summed over
// the pair's match counts (core/ctmc.py:173-230, 285-326):
//   W[i]   = sum_ab n[a,b] I[a,b,i,i] / P_ab(t)
//   U[i,j] = Q[i,j] sum_ab n[a,b] I[a,b,i,j] / P_ab(t)   (zero diagonal)
// The reference builds the A^4 integral tensor I; with the symmetrised rate
// matrix D^1/2 Q D^-1/2 = V diag(lam) V^T (D = diag(pi)) the same sums are
// S = D^1/2 V (J o (V^T R V)) V^T D^-1/2, with R[a,b] = n[a,b] / P_ab(t)
// sqrt(pi_b / pi_a) and J[k,l] = (e^{lam_k t} - e^{lam_l t}) / (lam_k - lam_l)
// (t e^{lam_k t} where |lam_k - lam_l| < 1e-10, the reference's rule), so
// W = diag S and U = Q o S: four A^3 products per (pair, class) instead of
// an A^4 tensor.  The eigendecomposition is a property of the class, not of
// the pair: it is computed on the host once per rate matrix (cyclic Jacobi)
// and passed by value.
namespace pro {

constexpr int HR_MAXA = 32;
constexpr int HR_THREADS = 128;

struct HRClass {
    int A;
    double lam[HR_MAXA];
    double V[HR_MAXA * HR_MAXA];   // row-major, column k = eigenvector k
    double sp[HR_MAXA];            // sqrt(pi)
    double Q[HR_MAXA * HR_MAXA];
};

__device__ __forceinline__ void hr_kernel_body(const HRClass &hc, int c, int C, const double *__restrict__ t,
                                               const double *__restrict__ mc, double *__restrict__ W,
                                               double *__restrict__ U) {
    __shared__ double V[HR_MAXA * HR_MAXA], R[HR_MAXA * HR_MAXA], T1[HR_MAXA * HR_MAXA], Y[HR_MAXA * HR_MAXA];
    __shared__ double ex[HR_MAXA], lam[HR_MAXA], sp[HR_MAXA];
    const int p = blockIdx.x, tid = threadIdx.x, A = hc.A, AA = A * A;
    const double tp = t[p];
    for (int i = tid; i < AA; i += HR_THREADS) V[i] = hc.V[i];
    for (int i = tid; i < A; i += HR_THREADS) {
        lam[i] = hc.lam[i];
        sp[i] = hc.sp[i];
        ex[i] = exp(hc.lam[i] * tp);
    }
    __syncthreads();
    const size_t base = ((size_t)p * C + c) * AA;
    const double *n = mc + base;
    // R = n / P(t), P_ab(t) = sqrt(pi_b / pi_a) sum_k V[a,k] e^{lam_k t} V[b,k]
    for (int i = tid; i < AA; i += HR_THREADS) {
        const int a = i / A, b = i - a * A;
        double s = 0.0;
        for (int k = 0; k < A; ++k) s += V[a * A + k] * ex[k] * V[b * A + k];
        const double r = sp[b] / sp[a];
        const double Pab = s * r;
        R[i] = n[i] / (fabs(Pab) < 1e-30 ? 1.0 : Pab) * r;
    }
    __syncthreads();
    // T1 = V^T R
    for (int i = tid; i < AA; i += HR_THREADS) {
        const int k = i / A, b = i - k * A;
        double s = 0.0;
        for (int a = 0; a < A; ++a) s += V[a * A + k] * R[a * A + b];
        T1[i] = s;
    }
    __syncthreads();
    // Y = J o (T1 V)
    for (int i = tid; i < AA; i += HR_THREADS) {
        const int k = i / A, l = i - k * A;
        double s = 0.0;
        for (int b = 0; b < A; ++b) s += T1[k * A + b] * V[b * A + l];
        const double d = lam[k] - lam[l];
        const double j = fabs(d) < 1e-10 ? tp * ex[k] : (ex[k] - ex[l]) / d;
        Y[i] = j * s;
    }
    __syncthreads();
    // R = V Y
    for (int i = tid; i < AA; i += HR_THREADS) {
        const int a = i / A, l = i - a * A;
        double s = 0.0;
        for (int k = 0; k < A; ++k) s += V[a * A + k] * Y[k * A + l];
        R[i] = s;
    }
    __syncthreads();
    // S = D^1/2 (R V^T) D^-1/2; W = diag S, U = Q o S off the diagonal
    for (int i = tid; i < AA; i += HR_THREADS) {
        const int a = i / A, b = i - a * A;
        double s = 0.0;
        for (int l = 0; l < A; ++l) s += R[a * A + l] * V[b * A + l];
        s *= sp[a] / sp[b];
        U[base + i] = a == b ? 0.0 : hc.Q[i] * s;
        if (a == b) W[((size_t)p * C + c) * A + a] = s;
    }
}

__global__ void __launch_bounds__(HR_THREADS) hr_kernel(const __grid_constant__ HRClass hc, int c, int C,
                                                        const double *__restrict__ t,
                                                        const double *__restrict__ mc, double *__restrict__ W,
                                                        double *__restrict__ U) {
    hr_kernel_body(hc, c, C, t, mc, W, U);
}

// the same with the class blocks in device memory (hcs[c]; a captured graph
// refreshes them by a copy before each replay)
__global__ void __launch_bounds__(HR_THREADS) hr_kernel_dp(const HRClass *__restrict__ hcs, int c, int C,
                                                           const double *__restrict__ t,
                                                           const double *__restrict__ mc, double *__restrict__ W,
                                                           double *__restrict__ U) {
    hr_kernel_body(hcs[c], c, C, t, mc, W, U);
}

// Eigenvalues and orthonormal eigenvectors of a symmetric n x n matrix by the
// cyclic Jacobi method (Golub & Van Loan, Matrix Computations, sec. 8.5):
// sweeps of plane rotations, each zeroing one off-diagonal entry with the
// smaller rotation angle, until the off-diagonal mass is below roundoff.
// a is overwritten; v receives the eigenvectors as columns.
static void sym_eig_jacobi(int n, double *a, double *lam, double *v) {
    for (int i = 0; i < n * n; ++i) v[i] = 0.0;
    for (int i = 0; i < n; ++i) v[i * n + i] = 1.0;
    double total = 0.0;
    for (int i = 0; i < n * n; ++i) total += a[i] * a[i];
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += a[p * n + q] * a[p * n + q];
        if (off <= 1e-36 * total || off == 0.0) break;
        for (int p = 0; p < n; ++p) {
            for (int q = p + 1; q < n; ++q) {
                const double apq = a[p * n + q];
                if (apq == 0.0) continue;
                const double theta = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
                const double tn = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double cs = 1.0 / std::sqrt(tn * tn + 1.0), sn = tn * cs;
                for (int k = 0; k < n; ++k) {   // columns p, q
                    const double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = cs * akp - sn * akq;
                    a[k * n + q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < n; ++k) {   // rows p, q
                    const double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = cs * apk - sn * aqk;
                    a[q * n + k] = sn * apk + cs * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = v[k * n + p], vkq = v[k * n + q];
                    v[k * n + p] = cs * vkp - sn * vkq;
                    v[k * n + q] = sn * vkp + cs * vkq;
                }
            }
        }
    }
    for (int i = 0; i < n; ++i) lam[i] = a[i * n + i];
}

// The class-level part, cached by the exact rate matrix and frequencies (EM
// calls the E-step many times between parameter updates).
struct HRCacheEntry {
    std::vector<double> key;
    HRClass hc;
};
static std::mutex hr_mu;
static std::deque<HRCacheEntry> hr_cache;
constexpr size_t HR_CACHE = 32;

static void hr_class(int A, const double *Q, const double *pi, HRClass &hc) {
    std::vector<double> key(Q, Q + A * A);
    key.insert(key.end(), pi, pi + A);
    {
        std::lock_guard<std::mutex> g(hr_mu);
        for (const auto &e : hr_cache)
            if (e.key.size() == key.size() && std::memcmp(e.key.data(), key.data(), sizeof(double) * key.size()) == 0) {
                hc = e.hc;
                return;
            }
    }
    std::memset(&hc, 0, sizeof(hc));
    hc.A = A;
    for (int a = 0; a < A; ++a) hc.sp[a] = std::sqrt(pi[a]);
    std::vector<double> sym(A * A);
    for (int a = 0; a < A; ++a)
        for (int b = 0; b < A; ++b) {
            const double x = Q[a * A + b] * (hc.sp[a] / hc.sp[b]);
            const double y = Q[b * A + a] * (hc.sp[b] / hc.sp[a]);
            sym[a * A + b] = 0.5 * (x + y);
        }
    std::vector<double> v(A * A);
    sym_eig_jacobi(A, sym.data(), hc.lam, v.data());
    std::memcpy(hc.V, v.data(), sizeof(double) * A * A);
    std::memcpy(hc.Q, Q, sizeof(double) * A * A);
    std::lock_guard<std::mutex> g(hr_mu);
    hr_cache.push_front(HRCacheEntry{std::move(key), hc});
    if (hr_cache.size() > HR_CACHE) hr_cache.pop_back();
}

}  // namespace pro

extern "C" int phmm_holmes_rubin(int32_t n_classes, int32_t alphabet, const double *class_Q, const double *class_pis,
                                 int32_t n_pairs, const double *t, const double *class_match_counts, double *W,
                                 double *U, void *stream) {
    using namespace pro;
    if (n_classes < 1 || alphabet < 1 || alphabet > HR_MAXA)
        return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin: need n_classes >= 1 and 1 <= alphabet <= 32");
    if (!class_Q || !class_pis) return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin: null host rate matrices");
    if (n_pairs < 0) return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin: negative n_pairs");
    for (int i = 0; i < n_classes * alphabet; ++i)
        if (!(class_pis[i] > 0.0))
            return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin: stationary frequencies must be positive");
    if (n_pairs == 0) return PHMM_OK;
    if (!t || !class_match_counts || !W || !U) return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin: null device buffer");
    const int A = alphabet;
    for (int c = 0; c < n_classes; ++c) {
        HRClass hc;
        hr_class(A, class_Q + (size_t)c * A * A, class_pis + (size_t)c * A, hc);
        hr_kernel<<<n_pairs, HR_THREADS, 0, (cudaStream_t)stream>>>(hc, c, n_classes, t, class_match_counts, W, U);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

// ---------------------------------------------------------------- parameter blocks in device memory
// For a captured CUDA graph of the batched E-step: the by-value parameter
// blocks above are baked into a graph's kernel nodes when it is captured, so
// the graph's kernels take them from device memory instead, refreshed before
// each replay by a copy from a host block that these functions fill.

extern "C" size_t phmm_mixdom2_param_block_bytes(void) { return sizeof(pro::Packed); }

extern "C" int phmm_mixdom2_param_block(const phmm_mixdom2_params *prm, void *host_block, size_t bytes) {
    using namespace pro;
    if (!host_block || bytes < sizeof(Packed))
        return pro_fail(PHMM_E_ARG, "phmm_mixdom2_param_block: host block missing or smaller than "
                                    "phmm_mixdom2_param_block_bytes()");
    return pack_params(prm, *reinterpret_cast<Packed *>(host_block), "phmm_mixdom2_param_block");
}

static int mixdom2_tables_dp(const void *param_block, int32_t n_dom, int32_t n_frag, int32_t n_classes,
                             int32_t n_pairs, const double *t, float *chi, float *emit_M, float *emit_I,
                             float *emit_D, double *class_subs, float *nest, void *stream);

extern "C" int phmm_mixdom2_tables_dp(const void *param_block, int32_t n_dom, int32_t n_frag, int32_t n_classes,
                                      int32_t n_pairs, const double *t, float *chi, float *emit_M, float *emit_I,
                                      float *emit_D, double *class_subs, void *stream) {
    return mixdom2_tables_dp(param_block, n_dom, n_frag, n_classes, n_pairs, t, chi, emit_M, emit_I, emit_D,
                             class_subs, nullptr, stream);
}

extern "C" int phmm_mixdom2_tables_nest_dp(const void *param_block, int32_t n_dom, int32_t n_frag,
                                           int32_t n_classes, int32_t n_pairs, const double *t, float *chi,
                                           float *emit_M, float *emit_I, float *emit_D, double *class_subs,
                                           float *nest, void *stream) {
    if (!nest && n_pairs > 0) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_tables_nest_dp: null nest buffer");
    return mixdom2_tables_dp(param_block, n_dom, n_frag, n_classes, n_pairs, t, chi, emit_M, emit_I, emit_D,
                             class_subs, nest, stream);
}

static int mixdom2_tables_dp(const void *param_block, int32_t n_dom, int32_t n_frag, int32_t n_classes,
                             int32_t n_pairs, const double *t, float *chi, float *emit_M, float *emit_I,
                             float *emit_D, double *class_subs, float *nest, void *stream) {
    using namespace pro;
    const int K = n_dom, F = n_frag, C = n_classes;
    if (K < 1 || F < 1 || C < 1 || K * F > MAXK || n_pairs < 0)
        return pro_fail(PHMM_E_ARG, "phmm_mixdom2_tables_dp: bad shape");
    if (n_pairs == 0) return PHMM_OK;
    if (!param_block || !t || !chi || !emit_M || !emit_I || !emit_D || !class_subs)
        return pro_fail(PHMM_E_ARG, "phmm_mixdom2_tables_dp: null device buffer");
    const Packed *pk = reinterpret_cast<const Packed *>(param_block);
    const int N = 2 + 5 * K * F;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t chi_smem = sizeof(double) * ChiSmem<double>::elems(K);
    if (chi_smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(chi_kernel_dp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)chi_smem);
        if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    }
    chi_kernel_dp<<<n_pairs, THREADS, chi_smem, st>>>(pk, t, N, chi, nullptr, nest);
    expm_kernel_dp<<<n_pairs * C, THREADS, 0, st>>>(pk, t, class_subs);
    tables_kernel_dp<<<n_pairs, THREADS, 0, st>>>(pk, class_subs, emit_M, emit_I, emit_D);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

extern "C" int phmm_mixdom2_nest(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t, float *nest,
                                 void *stream) {
    using namespace pro;
    Packed pk;
    int rc = pack_params(prm, pk, "phmm_mixdom2_nest");
    if (rc) return rc;
    if (n_pairs < 0) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_nest: negative n_pairs");
    if (n_pairs == 0) return PHMM_OK;
    if (!t || !nest) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_nest: null device buffer");
    const int N = 2 + 5 * pk.K * pk.F;
    const size_t chi_smem = sizeof(double) * ChiSmem<double>::elems(pk.K);
    if (chi_smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(nest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)chi_smem);
        if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    }
    nest_kernel<<<n_pairs, THREADS, chi_smem, (cudaStream_t)stream>>>(pk, t, N, nest);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

extern "C" int phmm_mixdom2_nest_dp(const void *param_block, int32_t n_dom, int32_t n_frag, int32_t n_classes,
                                    int32_t n_pairs, const double *t, float *nest, void *stream) {
    using namespace pro;
    const int K = n_dom, F = n_frag, C = n_classes;
    if (K < 1 || F < 1 || C < 1 || K * F > MAXK || n_pairs < 0)
        return pro_fail(PHMM_E_ARG, "phmm_mixdom2_nest_dp: bad shape");
    if (n_pairs == 0) return PHMM_OK;
    if (!param_block || !t || !nest) return pro_fail(PHMM_E_ARG, "phmm_mixdom2_nest_dp: null device buffer");
    const Packed *pk = reinterpret_cast<const Packed *>(param_block);
    const int N = 2 + 5 * K * F;
    const size_t chi_smem = sizeof(double) * ChiSmem<double>::elems(K);
    if (chi_smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(nest_kernel_dp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)chi_smem);
        if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    }
    nest_kernel_dp<<<n_pairs, THREADS, chi_smem, (cudaStream_t)stream>>>(pk, t, N, nest);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

extern "C" int phmm_mixdom2_class_counts_dp(const void *param_block, int32_t n_dom, int32_t n_frag,
                                            int32_t n_classes, int32_t n_pairs, const double *class_subs,
                                            const double *cnt_M, const double *cnt_I, const double *cnt_D,
                                            double *class_match, double *class_insert, double *class_delete,
                                            double *classdist_counts, void *stream) {
    using namespace pro;
    const int K = n_dom, F = n_frag, C = n_classes;
    if (K < 1 || F < 1 || C < 1 || K * F > MAXK || C > CS_MAXC || n_pairs < 0)
        return pro_fail(PHMM_E_ARG, "phmm_mixdom2_class_counts_dp: bad shape (at most 8 classes)");
    if (n_pairs == 0) return PHMM_OK;
    if (!param_block || !class_subs || !cnt_M || !cnt_I || !cnt_D || !class_match || !class_insert ||
        !class_delete || !classdist_counts)
        return pro_fail(PHMM_E_ARG, "phmm_mixdom2_class_counts_dp: null device buffer");
    const size_t smem = sizeof(double) * K * F * C;
    class_split_kernel_dp<<<n_pairs, THREADS, smem, (cudaStream_t)stream>>>(
        reinterpret_cast<const Packed *>(param_block), class_subs, cnt_M, cnt_I, cnt_D, class_match, class_insert,
        class_delete, classdist_counts);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

extern "C" size_t phmm_holmes_rubin_block_bytes(int32_t n_classes) {
    return n_classes > 0 ? sizeof(pro::HRClass) * (size_t)n_classes : 0;
}

extern "C" int phmm_holmes_rubin_block(int32_t n_classes, int32_t alphabet, const double *class_Q,
                                       const double *class_pis, void *host_block, size_t bytes) {
    using namespace pro;
    if (n_classes < 1 || alphabet < 1 || alphabet > HR_MAXA)
        return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin_block: need n_classes >= 1 and 1 <= alphabet <= 32");
    if (!class_Q || !class_pis) return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin_block: null host rate matrices");
    if (!host_block || bytes < sizeof(HRClass) * (size_t)n_classes)
        return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin_block: host block smaller than phmm_holmes_rubin_block_bytes");
    for (int i = 0; i < n_classes * alphabet; ++i)
        if (!(class_pis[i] > 0.0))
            return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin_block: stationary frequencies must be positive");
    HRClass *out = reinterpret_cast<HRClass *>(host_block);
    const int A = alphabet;
    for (int c = 0; c < n_classes; ++c) hr_class(A, class_Q + (size_t)c * A * A, class_pis + (size_t)c * A, out[c]);
    return PHMM_OK;
}

extern "C" int phmm_holmes_rubin_dp(const void *block, int32_t n_classes, int32_t n_pairs, const double *t,
                                    const double *class_match_counts, double *W, double *U, void *stream) {
    using namespace pro;
    if (n_classes < 1 || n_pairs < 0) return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin_dp: bad shape");
    if (n_pairs == 0) return PHMM_OK;
    if (!block || !t || !class_match_counts || !W || !U)
        return pro_fail(PHMM_E_ARG, "phmm_holmes_rubin_dp: null device buffer");
    for (int c = 0; c < n_classes; ++c)
        hr_kernel_dp<<<n_pairs, HR_THREADS, 0, (cudaStream_t)stream>>>(reinterpret_cast<const HRClass *>(block), c,
                                                                       n_classes, t, class_match_counts, W, U);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pro_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}
