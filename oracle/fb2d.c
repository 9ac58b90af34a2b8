/* FP64 oracle in C: 2D pair-HMM forward-backward (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle's fast twin of oracle/dp.py, used by the test-suite (against
 * the NumPy oracle) and by bench.py's CPU legs; the product never links it.
 * It restates the same log-space recursions of the reference
 * (python/tkfmixdom/jax/dp/hmm.py):
 *   forward  (dp/hmm.py:1120-1292): F[0,0,S] = 0; for M/I/D destination k at
 *            (i, j), F = lse_s(F[pred_k, s] + logT[s, k]) + e[i, j, k] with
 *            pred M (i-1, j-1), I (i, j-1), D (i-1, j); S/E destinations and
 *            missing predecessors NEG_INF; LL = lse_s(F[Lx, Ly, s] + logT[s, E]);
 *   backward (dp/hmm.py:1295-1437, 1695-1772): B[Lx, Ly, s] = logT[s, E];
 *            elsewhere B[i, j, s] = lse over M/I/D successors k of
 *            logT[s, k] + e[succ_k, k] + B[succ_k, k];
 *   counts   (dp/hmm.py:1940-1971): n[s, k] = sum over cells of
 *            exp(F[src, s] + logT[s, k] + e[dst, k] + B[dst, k] - LL), plus
 *            n[s, E] += exp(F[Lx, Ly, s] + logT[s, E] - LL).
 * NEG_INF is -1e30 and is summed like any other number, as the reference does.
 * Cells in anti-diagonal order.  The cells of one anti-diagonal are
 * independent, so with OpenMP (oracle/build_oracle.py builds with -fopenmp
 * where the compiler has it) they run on oracle_set_threads() host threads;
 * each cell's arithmetic is the same as in the serial loop, and the count
 * sums are per-thread partials added in thread order.  The tables are
 * caller-owned; only the per-thread count partials are allocated here. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NEG_INF (-1e30)

enum { TS = 0, TM = 1, TI = 2, TD = 3, TE = 4 };

/* Host threads of the following calls (1 = serial); returns the number in use. */
int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

static double lse(const double *v, int n) {
    double m = v[0];
    for (int k = 1; k < n; ++k)
        if (v[k] > m) m = v[k];
    double s = 0.0;
    for (int k = 0; k < n; ++k) s += exp(v[k] - m);
    return m + log(s);
}

/* F, B: (Lx+1)(Ly+1)N doubles each (B unused when forward_only); tmp: N
 * doubles.  Returns the log-likelihood; n_trans (N*N, zeroed here) may be
 * NULL when forward_only. */
double oracle_fb2d(int N, const int8_t *st, const double *lt, int Lx, int Ly, const double *emit,
                   int forward_only, double *F, double *B, double *n_trans, double *tmp) {
    const int W = Ly + 1;
    int e_idx = 0;
    for (int k = 0; k < N; ++k)
        if (st[k] == TE) { e_idx = k; break; }
#define AT(T, i, j) ((T) + ((size_t)(i) * W + (size_t)(j)) * (size_t)N)
    for (size_t q = 0; q < (size_t)(Lx + 1) * W * N; ++q) F[q] = NEG_INF;
    F[0] = 0.0;   /* state 0 is the start */
    for (int d = 1; d <= Lx + Ly; ++d) {
        const int ilo = d - Ly > 0 ? d - Ly : 0, ihi = d < Lx ? d : Lx;
#pragma omp parallel for schedule(static) if (ihi - ilo >= 32)
        for (int i = ilo; i <= ihi; ++i) {
            double tv[N];
            const int j = d - i;
            double *out = AT(F, i, j);
            const double *e = AT(emit, i, j);
            for (int k = 0; k < N; ++k) {
                const double *pred = NULL;
                if (st[k] == TM && i >= 1 && j >= 1) pred = AT(F, i - 1, j - 1);
                else if (st[k] == TI && j >= 1) pred = AT(F, i, j - 1);
                else if (st[k] == TD && i >= 1) pred = AT(F, i - 1, j);
                if (!pred) { out[k] = NEG_INF; continue; }
                for (int s = 0; s < N; ++s) tv[s] = pred[s] + lt[s * N + k];
                out[k] = lse(tv, N) + e[k];
            }
        }
    }
    const double *last = AT(F, Lx, Ly);
    for (int s = 0; s < N; ++s) tmp[s] = last[s] + lt[s * N + e_idx];
    const double ll = lse(tmp, N);
    if (forward_only) return ll;
    for (size_t q = 0; q < (size_t)(Lx + 1) * W * N; ++q) B[q] = NEG_INF;
    for (int s = 0; s < N; ++s) AT(B, Lx, Ly)[s] = lt[s * N + e_idx];
    for (int d = Lx + Ly - 1; d >= 0; --d) {
        const int ilo = d - Ly > 0 ? d - Ly : 0, ihi = d < Lx ? d : Lx;
#pragma omp parallel for schedule(static) if (ihi - ilo >= 32)
        for (int i = ilo; i <= ihi; ++i) {
            double tv[N];
            const int j = d - i;
            double *out = AT(B, i, j);
            for (int s = 0; s < N; ++s) {
                int n = 0;
                for (int k = 0; k < N; ++k) {
                    int ni, nj;
                    if (st[k] == TM) { ni = i + 1; nj = j + 1; }
                    else if (st[k] == TI) { ni = i; nj = j + 1; }
                    else if (st[k] == TD) { ni = i + 1; nj = j; }
                    else continue;
                    if (ni > Lx || nj > Ly) continue;
                    tv[n++] = lt[s * N + k] + AT(emit, ni, nj)[k] + AT(B, ni, nj)[k];
                }
                out[s] = n ? lse(tv, n) : NEG_INF;
            }
        }
    }
    memset(n_trans, 0, sizeof(double) * (size_t)N * N);
    int nth = 1;
#ifdef _OPENMP
    nth = (Lx + 1) * (Ly + 1) >= 4096 ? omp_get_max_threads() : 1;
#endif
    double *part = nth > 1 ? (double *)calloc((size_t)nth * N * N, sizeof(double)) : NULL;
    if (!part) nth = 1;
#pragma omp parallel num_threads(nth) if (nth > 1)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *acc = nth > 1 ? part + (size_t)tid * N * N : n_trans;
#pragma omp for schedule(static)
        for (int i = 0; i <= Lx; ++i)
            for (int j = 0; j <= Ly; ++j) {
                const double *f = AT(F, i, j);
                for (int k = 0; k < N; ++k) {
                    int ni, nj;
                    if (st[k] == TM) { ni = i + 1; nj = j + 1; }
                    else if (st[k] == TI) { ni = i; nj = j + 1; }
                    else if (st[k] == TD) { ni = i + 1; nj = j; }
                    else continue;
                    if (ni > Lx || nj > Ly) continue;
                    const double w = AT(emit, ni, nj)[k] + AT(B, ni, nj)[k] - ll;
                    for (int s = 0; s < N; ++s) acc[s * N + k] += exp(f[s] + lt[s * N + k] + w);
                }
            }
    }
    if (nth > 1) {
        for (int t = 0; t < nth; ++t)
            for (size_t q = 0; q < (size_t)N * N; ++q) n_trans[q] += part[(size_t)t * N * N + q];
        free(part);
    }
    for (int s = 0; s < N; ++s) n_trans[s * N + e_idx] += exp(last[s] + lt[s * N + e_idx] - ll);
#undef AT
    return ll;
}

/* Per-group character counts of the posteriors (the kernels' native emission
 * counts; oracle/estep.py char_count_tables): for M states at i, j >= 1
 * cM[g][x_i][y_j] += post, for I states at j >= 1 cI[g][y_j] += post, for D
 * states at i >= 1 cD[g][x_i] += post, post = exp(F + B - LL).  xg / yg are
 * the grid characters (index 0 the dummy character), 0..20.  cM (G*441), cI
 * and cD (G*21) are zeroed here.  F and B as oracle_fb2d left them. */
void oracle_char_counts(int N, const int8_t *st, const int32_t *groups, int G, int Lx, int Ly,
                        const int32_t *xg, const int32_t *yg, const double *F, const double *B, double ll,
                        double *cM, double *cI, double *cD) {
    const int W = Ly + 1;
    memset(cM, 0, sizeof(double) * (size_t)G * 441);
    memset(cI, 0, sizeof(double) * (size_t)G * 21);
    memset(cD, 0, sizeof(double) * (size_t)G * 21);
    for (int i = 0; i <= Lx; ++i)
        for (int j = 0; j <= Ly; ++j) {
            const double *f = F + ((size_t)i * W + (size_t)j) * (size_t)N;
            const double *b = B + ((size_t)i * W + (size_t)j) * (size_t)N;
            for (int k = 0; k < N; ++k) {
                const int g = groups[k];
                if (st[k] == TM && i >= 1 && j >= 1) cM[(size_t)g * 441 + xg[i] * 21 + yg[j]] += exp(f[k] + b[k] - ll);
                else if (st[k] == TI && j >= 1) cI[(size_t)g * 21 + yg[j]] += exp(f[k] + b[k] - ll);
                else if (st[k] == TD && i >= 1) cD[(size_t)g * 21 + xg[i]] += exp(f[k] + b[k] - ll);
            }
        }
}
