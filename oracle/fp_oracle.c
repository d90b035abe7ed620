/*
 * fp_oracle.c -- CPU oracle for the Pauli apply / expectation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is compiled and
 * called by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
 * leg.  No product code path may link or call it.
 *
 * It restates, in plain C with OpenMP, the algorithms of the reference
 * (qognitive/fast-pauli, header-only C++):
 *
 *   fpo_sparse_repr        <- get_sparse_repr            fast_pauli/cpp/include/__pauli_string.hpp:49-118
 *   fpo_string_apply_batch <- PauliString::apply_batch   __pauli_string.hpp:378-436 (seq branch :425-434)
 *   fpo_string_expectation <- PauliString::expectation_value __pauli_string.hpp:471-538 (seq branch :529-537)
 *   fpo_op_apply           <- PauliOp::apply (par)       fast_pauli/cpp/include/__pauli_op.hpp:414-468
 *   fpo_op_expectation     <- PauliOp::expectation_value (par) __pauli_op.hpp:496-549
 *   fpo_summed_expectation <- SummedPauliOp::expectation_value (par) __summed_pauli_op.hpp:530-614
 *   fpo_summed_apply       <- SummedPauliOp::apply (par) __summed_pauli_op.hpp:287-349
 *   fpo_summed_apply_weighted <- SummedPauliOp::apply_weighted (par) __summed_pauli_op.hpp:378-503
 *
 * Loop structure (strings outer and OpenMP-parallel, the sparse pattern
 * rebuilt per string per call, per-thread output buffers reduced at the end)
 * follows the reference so that its timing is representative of the
 * reference's OpenMP "par" path.  Arithmetic is complex128 held as
 * interleaved (re, im) doubles.
 *
 * Pauli codes: 0 = I, 1 = X, 2 = Y, 3 = Z (__pauli.hpp:41).  A string of n
 * codes is given leftmost character first; the leftmost character acts on the
 * most significant bit of the row index (the reference reverses the view,
 * __pauli_string.hpp:54).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int thread_num(void)
{
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

/* complex helpers on (re, im) pairs */
static inline void cmul(double ar, double ai, double br, double bi, double *cr, double *ci)
{
    *cr = ar * br - ai * bi;
    *ci = ar * bi + ai * br;
}

/*
 * Sparse pattern of one Pauli string: column k[i] and value m[i] (re, im) of
 * the single non-zero entry in row i.  Restates the doubling construction of
 * get_sparse_repr (__pauli_string.hpp:49-118): row 0 is seeded with the
 * bit pattern of X/Y factors and the phase (-i)^{#Y}; block [2^l, 2^{l+1})
 * is derived from block [0, 2^l) by flipping column bit l for X/Y and
 * negating the value for Y/Z.
 */
void fpo_sparse_repr(const uint8_t *codes, int n, uint64_t *k, double *m)
{
    if (n <= 0)
        return;
    const uint64_t dim = (uint64_t)1 << n;
    int ny = 0;
    for (int j = 0; j < n; ++j)
        ny += codes[j] == 2;
    /* ps[l] = codes[n-1-l]  (reversed view) */
    uint64_t k0 = 0;
    for (int l = 0; l < n; ++l)
    {
        uint8_t c = codes[n - 1 - l];
        uint64_t diag = (c == 1 || c == 2) ? 1u : 0u;
        k0 += ((uint64_t)1 << l) * diag;
    }
    k[0] = k0;
    switch (ny % 4)
    {
    case 0: m[0] = 1.0; m[1] = 0.0; break;
    case 1: m[0] = 0.0; m[1] = -1.0; break;
    case 2: m[0] = -1.0; m[1] = 0.0; break;
    default: m[0] = 0.0; m[1] = 1.0; break;
    }
    for (int l = 0; l < n; ++l)
    {
        uint8_t c = codes[n - 1 - l];
        double eps = (c == 2 || c == 3) ? -1.0 : 1.0;
        int flip = (c == 1 || c == 2);
        uint64_t lb = (uint64_t)1 << l;
        for (uint64_t li = lb; li < (lb << 1); ++li)
        {
            k[li] = flip ? k[li - lb] - lb : k[li - lb] + lb;
            m[2 * li] = m[2 * (li - lb)] * eps;
            m[2 * li + 1] = m[2 * (li - lb) + 1] * eps;
        }
    }
    (void)dim;
}

/* new(i,t) += c * m[i] * psi(k[i], t)   -- seq branch of apply_batch */
void fpo_string_apply_batch(const uint8_t *codes, int n, int64_t S, const double *psi, double *out, double cr,
                            double ci)
{
    const uint64_t D = (uint64_t)1 << n;
    uint64_t *k = (uint64_t *)malloc(D * sizeof(uint64_t));
    double *m = (double *)malloc(2 * D * sizeof(double));
    fpo_sparse_repr(codes, n, k, m);
    for (uint64_t i = 0; i < D; ++i)
    {
        double cmr, cmi;
        cmul(cr, ci, m[2 * i], m[2 * i + 1], &cmr, &cmi);
        const double *row = psi + 2 * (k[i] * (uint64_t)S);
        double *o = out + 2 * (i * (uint64_t)S);
        for (int64_t t = 0; t < S; ++t)
        {
            double pr, pi;
            cmul(cmr, cmi, row[2 * t], row[2 * t + 1], &pr, &pi);
            o[2 * t] += pr;
            o[2 * t + 1] += pi;
        }
    }
    free(k);
    free(m);
}

/* ev[t] += conj(psi(i,t)) * c * m[i] * psi(k[i],t)  -- seq branch of expectation_value */
void fpo_string_expectation(const uint8_t *codes, int n, int64_t S, const double *psi, double *ev, double cr,
                            double ci)
{
    const uint64_t D = (uint64_t)1 << n;
    uint64_t *k = (uint64_t *)malloc(D * sizeof(uint64_t));
    double *m = (double *)malloc(2 * D * sizeof(double));
    fpo_sparse_repr(codes, n, k, m);
    for (uint64_t i = 0; i < D; ++i)
    {
        double cmr, cmi;
        cmul(cr, ci, m[2 * i], m[2 * i + 1], &cmr, &cmi);
        const double *a = psi + 2 * (i * (uint64_t)S);
        const double *b = psi + 2 * (k[i] * (uint64_t)S);
        for (int64_t t = 0; t < S; ++t)
        {
            double ur, ui, vr, vi;
            cmul(a[2 * t], -a[2 * t + 1], cmr, cmi, &ur, &ui);
            cmul(ur, ui, b[2 * t], b[2 * t + 1], &vr, &vi);
            ev[2 * t] += vr;
            ev[2 * t + 1] += vi;
        }
    }
    free(k);
    free(m);
}

/*
 * PauliOp::apply, par: strings split statically over threads, each thread
 * accumulating into its own full (D,S) buffer, then a reduction over threads
 * (__pauli_op.hpp:427-456).  out += sum_j coeffs[j] P_j psi.
 */
void fpo_op_apply(const uint8_t *codes, int64_t P, int n, const double *coeffs, int64_t S, const double *psi,
                  double *out)
{
    const uint64_t D = (uint64_t)1 << n;
    const int nt = max_threads();
    const size_t blk = (size_t)D * (size_t)S * 2;
    double *thr = (double *)calloc((size_t)nt * blk, sizeof(double));
#pragma omp parallel
    {
        double *local = thr + (size_t)thread_num() * blk;
#pragma omp for schedule(static)
        for (int64_t j = 0; j < P; ++j)
            fpo_string_apply_batch(codes + j * n, n, S, psi, local, coeffs[2 * j], coeffs[2 * j + 1]);
#pragma omp for schedule(static)
        for (int64_t e = 0; e < (int64_t)(D * (uint64_t)S); ++e)
            for (int th = 0; th < nt; ++th)
            {
                out[2 * e] += thr[(size_t)th * blk + 2 * e];
                out[2 * e + 1] += thr[(size_t)th * blk + 2 * e + 1];
            }
    }
    free(thr);
}

/* PauliOp::expectation_value, par (__pauli_op.hpp:509-538). ev (S,) += sum_j c_j <P_j> */
void fpo_op_expectation(const uint8_t *codes, int64_t P, int n, const double *coeffs, int64_t S, const double *psi,
                        double *ev)
{
    const int nt = max_threads();
    double *thr = (double *)calloc((size_t)nt * (size_t)S * 2, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < P; ++j)
        fpo_string_expectation(codes + j * n, n, S, psi, thr + (size_t)thread_num() * (size_t)S * 2,
                               coeffs[2 * j], coeffs[2 * j + 1]);
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < S; ++t)
        for (int th = 0; th < nt; ++th)
        {
            ev[2 * t] += thr[((size_t)th * S + t) * 2];
            ev[2 * t + 1] += thr[((size_t)th * S + t) * 2 + 1];
        }
    free(thr);
}

/*
 * SummedPauliOp::expectation_value, par (__summed_pauli_op.hpp:567-592):
 * per-string expectation values (P,S) with strings split over threads, then
 * out(k,t) += sum_j h(j,k) * ev(j,t) collapsed over (k,t).
 * h is row-major (P, K); out is (K, S).
 */
void fpo_summed_expectation(const uint8_t *codes, int64_t P, int n, const double *h, int64_t K, int64_t S,
                            const double *psi, double *out)
{
    double *ev = (double *)calloc((size_t)P * (size_t)S * 2, sizeof(double));
#pragma omp parallel
    {
#pragma omp for schedule(static)
        for (int64_t j = 0; j < P; ++j)
            fpo_string_expectation(codes + j * n, n, S, psi, ev + (size_t)j * (size_t)S * 2, 1.0, 0.0);
#pragma omp for collapse(2) schedule(static)
        for (int64_t k = 0; k < K; ++k)
            for (int64_t t = 0; t < S; ++t)
            {
                double ar = 0.0, ai = 0.0;
                for (int64_t j = 0; j < P; ++j)
                {
                    double pr, pi;
                    cmul(h[2 * (j * K + k)], h[2 * (j * K + k) + 1], ev[2 * (j * S + t)], ev[2 * (j * S + t) + 1],
                         &pr, &pi);
                    ar += pr;
                    ai += pi;
                }
                out[2 * (k * S + t)] += ar;
                out[2 * (k * S + t) + 1] += ai;
            }
    }
    free(ev);
}

/* SummedPauliOp::apply, par (__summed_pauli_op.hpp:304-335): c_j = sum_k h(j,k), then PauliOp-style apply */
void fpo_summed_apply(const uint8_t *codes, int64_t P, int n, const double *h, int64_t K, int64_t S,
                      const double *psi, double *out)
{
    double *c = (double *)calloc((size_t)P * 2, sizeof(double));
    for (int64_t j = 0; j < P; ++j)
        for (int64_t k = 0; k < K; ++k)
        {
            c[2 * j] += h[2 * (j * K + k)];
            c[2 * j + 1] += h[2 * (j * K + k) + 1];
        }
    fpo_op_apply(codes, P, n, c, S, psi, out);
    free(c);
}

/*
 * SummedPauliOp::apply_weighted, par (__summed_pauli_op.hpp:406-468):
 * w(j,t) = sum_k h(j,k) * data(k,t)   (data real, (K,S))
 * out(:,t) += sum_j w(j,t) * (P_j psi)(:,t), via a per-thread temporary per string.
 */
void fpo_summed_apply_weighted(const uint8_t *codes, int64_t P, int n, const double *h, int64_t K, int64_t S,
                               const double *psi, const double *data, double *out)
{
    const uint64_t D = (uint64_t)1 << n;
    const int nt = max_threads();
    const size_t blk = (size_t)D * (size_t)S * 2;
    double *thr = (double *)calloc((size_t)nt * blk, sizeof(double));
    double *w = (double *)calloc((size_t)P * (size_t)S * 2, sizeof(double));
#pragma omp parallel
    {
#pragma omp for schedule(dynamic) collapse(2)
        for (int64_t j = 0; j < P; ++j)
            for (int64_t t = 0; t < S; ++t)
                for (int64_t k = 0; k < K; ++k)
                {
                    w[2 * (j * S + t)] += h[2 * (j * K + k)] * data[k * S + t];
                    w[2 * (j * S + t) + 1] += h[2 * (j * K + k) + 1] * data[k * S + t];
                }
        double *tmp = (double *)malloc(blk * sizeof(double));
        double *local = thr + (size_t)thread_num() * blk;
#pragma omp for schedule(dynamic)
        for (int64_t j = 0; j < P; ++j)
        {
            memset(tmp, 0, blk * sizeof(double));
            fpo_string_apply_batch(codes + j * n, n, S, psi, tmp, 1.0, 0.0);
            for (uint64_t l = 0; l < D; ++l)
                for (int64_t t = 0; t < S; ++t)
                {
                    double pr, pi;
                    size_t e = 2 * (l * (uint64_t)S + (uint64_t)t);
                    cmul(tmp[e], tmp[e + 1], w[2 * (j * S + t)], w[2 * (j * S + t) + 1], &pr, &pi);
                    local[e] += pr;
                    local[e + 1] += pi;
                }
        }
        free(tmp);
#pragma omp for schedule(static)
        for (int64_t e = 0; e < (int64_t)(D * (uint64_t)S); ++e)
            for (int th = 0; th < nt; ++th)
            {
                out[2 * e] += thr[(size_t)th * blk + 2 * e];
                out[2 * e + 1] += thr[(size_t)th * blk + 2 * e + 1];
            }
    }
    free(w);
    free(thr);
}

/*
 * Product of two Pauli matrices (codes 0..3): result code a ^ b and the phase
 * as a power of i -- the Pauli algebra XY = iZ, YZ = iX, ZX = iY (reversed
 * order: -i), as tabulated by Pauli::operator* (__pauli.hpp:109-175).
 */
static const int k_pow_i[4][4] = {{0, 0, 0, 0}, {0, 0, 1, 3}, {0, 3, 0, 1}, {0, 1, 3, 0}};

/* FNV-1a hash of a string of n codes (the reference keys a std::unordered_map
 * by PauliString, __summed_pauli_op.hpp:209-213) */
static uint64_t hash_codes(const uint8_t *c, int n)
{
    uint64_t hsh = 1469598103934665603ull;
    for (int q = 0; q < n; ++q)
        hsh = (hsh ^ c[q]) * 1099511628211ull;
    return hsh;
}

/*
 * fpo_summed_square <- SummedPauliOp::square (__summed_pauli_op.hpp:197-268),
 * products as PauliString::operator* (__pauli_string.hpp:228-247).
 * sq_codes: the A strings of the squared set (the caller passes
 * calculate_pauli_strings_max_weight(n, min(n, 2 w))); out: (A, K) complex,
 * overwritten.  Structure as the reference: an index map of the squared set
 * (later duplicates overwrite earlier ones), the per-output pair lists
 * t_aij built serially in (i, j) order, the coefficients transposed to (K, P),
 * then out(a, k) += (phase * h(i, k)) * h(j, k) in parallel over (a, k).
 * Returns 0, or -1 when a product is not in the set (the reference's map
 * would then send it to index 0).
 */
int fpo_summed_square(const uint8_t *codes, int64_t P, int n, const double *h, int64_t K, const uint8_t *sq_codes,
                      int64_t A, double *out)
{
    if (A <= 0 || K <= 0)
        return 0;
    memset(out, 0, (size_t)(A * K) * 2 * sizeof(double));
    if (P <= 0)
        return 0;
    /* open-addressing index map */
    int64_t cap = 1;
    while (cap < 2 * A)
        cap <<= 1;
    int64_t *slot = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
    for (int64_t s = 0; s < cap; ++s)
        slot[s] = -1;
    for (int64_t a = 0; a < A; ++a)
    {
        int64_t s = (int64_t)(hash_codes(sq_codes + a * n, n) & (uint64_t)(cap - 1));
        while (slot[s] >= 0 && memcmp(sq_codes + slot[s] * n, sq_codes + a * n, (size_t)n) != 0)
            s = (s + 1) & (cap - 1);
        slot[s] = a;
    }
    /* pair lists in CSR form: counts, then fill in (i, j) order */
    int64_t *cnt = (int64_t *)calloc((size_t)A + 1, sizeof(int64_t));
    int64_t *pidx = (int64_t *)malloc((size_t)(P * P) * sizeof(int64_t)); /* a of pair (i, j) */
    int8_t *pph = (int8_t *)malloc((size_t)(P * P));                      /* phase power of i */
    uint8_t *prod = (uint8_t *)malloc((size_t)n);
    int missing = 0;
    for (int64_t i = 0; i < P; ++i)
        for (int64_t j = 0; j < P; ++j)
        {
            int e = 0;
            for (int q = 0; q < n; ++q)
            {
                const uint8_t a = codes[i * n + q], b = codes[j * n + q];
                e += k_pow_i[a][b];
                prod[q] = (uint8_t)(a ^ b);
            }
            int64_t s = (int64_t)(hash_codes(prod, n) & (uint64_t)(cap - 1));
            while (slot[s] >= 0 && memcmp(sq_codes + slot[s] * n, prod, (size_t)n) != 0)
                s = (s + 1) & (cap - 1);
            int64_t a = slot[s];
            if (a < 0)
            {
                missing = 1;
                a = 0;
            }
            pidx[i * P + j] = a;
            pph[i * P + j] = (int8_t)(e & 3);
            cnt[a + 1]++;
        }
    for (int64_t a = 0; a < A; ++a)
        cnt[a + 1] += cnt[a];
    int64_t *fill = (int64_t *)malloc((size_t)A * sizeof(int64_t));
    memcpy(fill, cnt, (size_t)A * sizeof(int64_t));
    int64_t *ti = (int64_t *)malloc((size_t)(P * P) * sizeof(int64_t));
    int64_t *tj = (int64_t *)malloc((size_t)(P * P) * sizeof(int64_t));
    int8_t *tp = (int8_t *)malloc((size_t)(P * P));
    for (int64_t i = 0; i < P; ++i)
        for (int64_t j = 0; j < P; ++j)
        {
            const int64_t a = pidx[i * P + j];
            const int64_t x = fill[a]++;
            ti[x] = i;
            tj[x] = j;
            tp[x] = pph[i * P + j];
        }
    /* coefficients transposed to (K, P) */
    double *ht = (double *)malloc((size_t)(K * P) * 2 * sizeof(double));
    for (int64_t i = 0; i < P; ++i)
        for (int64_t k = 0; k < K; ++k)
        {
            ht[2 * (k * P + i)] = h[2 * (i * K + k)];
            ht[2 * (k * P + i) + 1] = h[2 * (i * K + k) + 1];
        }
    static const double ph_re[4] = {1, 0, -1, 0}, ph_im[4] = {0, 1, 0, -1};
#pragma omp parallel for schedule(dynamic) collapse(2)
    for (int64_t a = 0; a < A; ++a)
        for (int64_t k = 0; k < K; ++k)
        {
            double sr = 0, si = 0;
            for (int64_t x = cnt[a]; x < cnt[a + 1]; ++x)
            {
                double ar, ai, br, bi;
                const double *hi = ht + 2 * (k * P + ti[x]), *hj = ht + 2 * (k * P + tj[x]);
                cmul(ph_re[tp[x]], ph_im[tp[x]], hi[0], hi[1], &ar, &ai);
                cmul(ar, ai, hj[0], hj[1], &br, &bi);
                sr += br;
                si += bi;
            }
            out[2 * (a * K + k)] = sr;
            out[2 * (a * K + k) + 1] = si;
        }
    free(ht);
    free(tp);
    free(tj);
    free(ti);
    free(fill);
    free(prod);
    free(pph);
    free(pidx);
    free(cnt);
    free(slot);
    return missing ? -1 : 0;
}

/*
 * fpo_op_product <- PauliOp operator* (__pauli_op.hpp:237-281) with the
 * products of PauliString::operator* (__pauli_string.hpp:228-247): every
 * pair (i, j) in order, the product string position by position with the
 * Pauli table's phase, its coefficient phase * a_i * b_j added to the
 * string's entry in a hash map (one map, so equal strings always merge;
 * the reference keeps one map per OpenMP thread).  Writes the distinct
 * strings in order of first appearance to out_codes (n codes each) and
 * their coefficients to out_c (complex); both hold Pa * Pb entries.
 * Returns the number of distinct strings.
 */
int64_t fpo_op_product(const uint8_t *a_codes, const double *a_c, int64_t Pa, const uint8_t *b_codes,
                       const double *b_c, int64_t Pb, int n, uint8_t *out_codes, double *out_c)
{
    const int64_t N = Pa * Pb;
    if (N <= 0)
        return 0;
    int64_t cap = 1;
    while (cap < 2 * N)
        cap <<= 1;
    int64_t *slot = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
    for (int64_t s = 0; s < cap; ++s)
        slot[s] = -1;
    uint8_t *prod = (uint8_t *)malloc((size_t)(n > 0 ? n : 1));
    static const double ph_re[4] = {1, 0, -1, 0}, ph_im[4] = {0, 1, 0, -1};
    int64_t count = 0;
    for (int64_t i = 0; i < Pa; ++i)
        for (int64_t j = 0; j < Pb; ++j)
        {
            int e = 0;
            for (int q = 0; q < n; ++q)
            {
                const uint8_t x = a_codes[i * n + q], y = b_codes[j * n + q];
                e += k_pow_i[x][y];
                prod[q] = (uint8_t)(x ^ y);
            }
            double ar, ai, cr, ci;
            cmul(ph_re[e & 3], ph_im[e & 3], a_c[2 * i], a_c[2 * i + 1], &ar, &ai);
            cmul(ar, ai, b_c[2 * j], b_c[2 * j + 1], &cr, &ci);
            int64_t s = (int64_t)(hash_codes(prod, n) & (uint64_t)(cap - 1));
            while (slot[s] >= 0 && memcmp(out_codes + slot[s] * n, prod, (size_t)n) != 0)
                s = (s + 1) & (cap - 1);
            if (slot[s] < 0)
            {
                slot[s] = count;
                memcpy(out_codes + count * n, prod, (size_t)n);
                out_c[2 * count] = 0.0;
                out_c[2 * count + 1] = 0.0;
                ++count;
            }
            out_c[2 * slot[s]] += cr;
            out_c[2 * slot[s] + 1] += ci;
        }
    free(prod);
    free(slot);
    return count;
}

/*
 * fpo_summed_to_tensor <- SummedPauliOp::to_tensor (__summed_pauli_op.hpp:644-665):
 * out (K, D, D) complex, accumulated: for every string its sparse pattern,
 * then out(k, j, cols[j]) += h(i, k) * vals[j], strings in order, OpenMP over
 * the operators k.
 */
void fpo_summed_to_tensor(const uint8_t *codes, int64_t P, int n, const double *h, int64_t K, double *out)
{
    const uint64_t D = (uint64_t)1 << n;
    uint64_t *cols = (uint64_t *)malloc(D * sizeof(uint64_t));
    double *vals = (double *)malloc(D * 2 * sizeof(double));
    for (int64_t i = 0; i < P; ++i)
    {
        fpo_sparse_repr(codes + i * n, n, cols, vals);
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < K; ++k)
        {
            const double cr = h[2 * (i * K + k)], ci = h[2 * (i * K + k) + 1];
            for (uint64_t j = 0; j < D; ++j)
            {
                double vr, vi;
                cmul(cr, ci, vals[2 * j], vals[2 * j + 1], &vr, &vi);
                double *o = out + 2 * (((uint64_t)k * D + j) * D + cols[j]);
                o[0] += vr;
                o[1] += vi;
            }
        }
    }
    free(vals);
    free(cols);
}

int fpo_max_threads(void)
{
    return max_threads();
}
