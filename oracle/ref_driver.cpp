// ref_driver.cpp -- C-ABI driver over the reference's own C++ implementation.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh against the
// reference headers where they lie (fast_pauli/cpp/include, unmodified) into
// oracle/_ref/libfpref.so; used to pin the C restatement (fp_oracle.c) and to
// generate the golden fixtures in tests/golden/.  Never linked by product code.
//
// Every entry point calls the reference's std::execution::par overload, the
// one its Python bindings call (e.g. __pauli_op_bindings.hpp:497,506,
// __summed_pauli_op_bindings.hpp:173,219,265).  Complex arrays are interleaved
// (re, im) float64, row-major.  Outputs accumulate (+=), as in the reference.
#include <complex>
#include <cstdint>
#include <cstring>
#include <execution>
#include <string>
#include <vector>

#include "fast_pauli.hpp"

namespace fp = fast_pauli;
using cd = std::complex<double>;

template <size_t R> using Span = std::mdspan<cd, std::dextents<size_t, R>>;

static std::vector<fp::PauliString> parse(const char *strs, int64_t P, int n)
{
    std::vector<fp::PauliString> v;
    v.reserve(P);
    for (int64_t j = 0; j < P; ++j)
        v.emplace_back(std::string(strs + j * n, strs + (j + 1) * n));
    return v;
}

extern "C"
{

    int fpref_sparse_repr(const char *str, int n, uint64_t *cols, double *vals)
    {
        fp::PauliString ps(std::string(str, str + n));
        auto [k, m] = fp::get_sparse_repr<double>(ps.paulis);
        for (size_t i = 0; i < k.size(); ++i)
        {
            cols[i] = k[i];
            vals[2 * i] = m[i].real();
            vals[2 * i + 1] = m[i].imag();
        }
        return 0;
    }

    // PauliString.apply (2-D, honours coeff) -> apply_batch(par)
    int fpref_string_apply_batch(const char *str, int n, int64_t S, const double *psi, double *out, double cr,
                                 double ci)
    {
        fp::PauliString ps(std::string(str, str + n));
        size_t D = size_t(1) << n;
        Span<2> st((cd *)psi, D, (size_t)S), o((cd *)out, D, (size_t)S);
        ps.apply_batch(std::execution::par, o, st, cd(cr, ci));
        return 0;
    }

    // PauliString.apply (1-D): the binding ignores coeff (__pauli_string_bindings.hpp:142)
    int fpref_string_apply_1d(const char *str, int n, const double *psi, double *out)
    {
        fp::PauliString ps(std::string(str, str + n));
        size_t D = size_t(1) << n;
        Span<1> st((cd *)psi, D), o((cd *)out, D);
        ps.apply(std::execution::par, o, st);
        return 0;
    }

    int fpref_string_expectation(const char *str, int n, int64_t S, const double *psi, double *ev, double cr,
                                 double ci)
    {
        fp::PauliString ps(std::string(str, str + n));
        size_t D = size_t(1) << n;
        Span<2> st((cd *)psi, D, (size_t)S);
        Span<1> e((cd *)ev, (size_t)S);
        ps.expectation_value(std::execution::par, e, st, cd(cr, ci));
        return 0;
    }

    int fpref_op_apply(const char *strs, int64_t P, int n, const double *coeffs, int64_t S, const double *psi,
                       double *out)
    {
        std::vector<cd> c((cd *)coeffs, (cd *)coeffs + P);
        fp::PauliOp<double> op(c, parse(strs, P, n));
        size_t D = size_t(1) << n;
        Span<2> st((cd *)psi, D, (size_t)S), o((cd *)out, D, (size_t)S);
        op.apply(std::execution::par, o, st);
        return 0;
    }

    int fpref_op_expectation(const char *strs, int64_t P, int n, const double *coeffs, int64_t S,
                             const double *psi, double *ev)
    {
        std::vector<cd> c((cd *)coeffs, (cd *)coeffs + P);
        fp::PauliOp<double> op(c, parse(strs, P, n));
        size_t D = size_t(1) << n;
        Span<2> st((cd *)psi, D, (size_t)S);
        Span<1> e((cd *)ev, (size_t)S);
        op.expectation_value(std::execution::par, e, st);
        return 0;
    }

    int fpref_summed_expectation(const char *strs, int64_t P, int n, const double *h, int64_t K, int64_t S,
                                 const double *psi, double *out)
    {
        Span<2> hs((cd *)h, (size_t)P, (size_t)K);
        fp::SummedPauliOp<double> op(parse(strs, P, n), hs);
        size_t D = size_t(1) << n;
        Span<2> st((cd *)psi, D, (size_t)S), o((cd *)out, (size_t)K, (size_t)S);
        op.expectation_value(std::execution::par, o, st);
        return 0;
    }

    int fpref_summed_apply(const char *strs, int64_t P, int n, const double *h, int64_t K, int64_t S,
                           const double *psi, double *out)
    {
        Span<2> hs((cd *)h, (size_t)P, (size_t)K);
        fp::SummedPauliOp<double> op(parse(strs, P, n), hs);
        size_t D = size_t(1) << n;
        Span<2> st((cd *)psi, D, (size_t)S), o((cd *)out, D, (size_t)S);
        op.apply(std::execution::par, o, st);
        return 0;
    }

    int fpref_summed_apply_weighted(const char *strs, int64_t P, int n, const double *h, int64_t K, int64_t S,
                                    const double *psi, const double *data, double *out)
    {
        Span<2> hs((cd *)h, (size_t)P, (size_t)K);
        fp::SummedPauliOp<double> op(parse(strs, P, n), hs);
        size_t D = size_t(1) << n;
        Span<2> st((cd *)psi, D, (size_t)S), o((cd *)out, D, (size_t)S);
        std::mdspan<double, std::dextents<size_t, 2>> ds((double *)data, (size_t)K, (size_t)S);
        op.apply_weighted(std::execution::par, o, st, ds);
        return 0;
    }

    // calculate_pauli_strings_max_weight(n, w): writes count*n chars into buf (if non-null), returns count
    int64_t fpref_pauli_strings_max_weight(int n, int w, char *buf)
    {
        auto v = fp::calculate_pauli_strings_max_weight((size_t)n, (size_t)w);
        if (buf)
            for (size_t j = 0; j < v.size(); ++j)
                for (int q = 0; q < n; ++q)
                    buf[j * n + q] = "IXYZ"[v[j].paulis[q].code];
        return (int64_t)v.size();
    }

    // SummedPauliOp::square: returns the new string count; writes strings and (P2 x K) coeffs when buffers given
    // PauliOp operator* of the reference; with out_strs == nullptr only the
    // number of result terms (one entry per string per OpenMP thread map)
    int64_t fpref_op_product(const char *a_strs, const double *a_c, int64_t Pa, const char *b_strs,
                             const double *b_c, int64_t Pb, int n, char *out_strs, double *out_c)
    {
        std::vector<cd> ca((cd *)a_c, (cd *)a_c + Pa), cb((cd *)b_c, (cd *)b_c + Pb);
        fp::PauliOp<double> a(ca, parse(a_strs, Pa, n)), b(cb, parse(b_strs, Pb, n));
        auto r = a * b;
        if (out_strs)
            for (size_t j = 0; j < r.pauli_strings.size(); ++j)
                for (int q = 0; q < n; ++q)
                    out_strs[j * n + q] = "IXYZ"[r.pauli_strings[j].paulis[q].code];
        if (out_c)
            std::memcpy(out_c, r.coeffs.data(), r.coeffs.size() * sizeof(cd));
        return (int64_t)r.pauli_strings.size();
    }

    int64_t fpref_summed_square(const char *strs, int64_t P, int n, const double *h, int64_t K, char *out_strs,
                                double *out_h)
    {
        Span<2> hs((cd *)h, (size_t)P, (size_t)K);
        fp::SummedPauliOp<double> op(parse(strs, P, n), hs);
        auto sq = op.square();
        if (out_strs)
            for (size_t j = 0; j < sq.pauli_strings.size(); ++j)
                for (int q = 0; q < n; ++q)
                    out_strs[j * n + q] = "IXYZ"[sq.pauli_strings[j].paulis[q].code];
        if (out_h)
            std::memcpy(out_h, sq.coeffs_raw.data(), sq.coeffs_raw.size() * sizeof(cd));
        return (int64_t)sq.pauli_strings.size();
    }
}
