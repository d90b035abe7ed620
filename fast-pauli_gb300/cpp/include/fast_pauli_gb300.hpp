// fast_pauli_gb300.hpp -- C++ host API of the GB300 Pauli engine.
//
// A drop-in for the hot-path classes of the reference's header-only C++
// library (qognitive/fast-pauli, fast_pauli/cpp/include/fast_pauli.hpp):
// namespace fast_pauli, classes Pauli, PauliString, PauliOp<T,H>,
// SummedPauliOp<T>, the helpers and get_sparse_repr<T>, with the same member
// names, argument meaning, accumulate-into-output semantics and
// std::invalid_argument errors.  The hot methods (apply, apply_batch,
// expectation_value, apply_weighted) run on the GPU through the C ABI of
// libfpg.so (include/fpg.h); there is no CPU fallback.
//
// Array arguments: any mdspan-like view (data_handle(), extent(r), rank()),
// e.g. std::mdspan / cuda::std::mdspan / fast_pauli::Span, of
// std::complex<double> (float64 path) or std::complex<float> (mixed path).
// Host arrays are staged to the device inside the call; device arrays (e.g.
// from cudaMalloc) are used in place.  The std::execution policy overloads
// are accepted for source compatibility; every call runs on the GPU.
#pragma once

#include <algorithm>
#include <array>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <execution>
#include <functional>
#include <initializer_list>
#include <memory>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "fpg.h"

namespace fast_pauli
{

// ---------------------------------------------------------------------------
// type traits (reference: __type_traits.hpp:26-53)
// ---------------------------------------------------------------------------
template <typename T> struct is_complex : std::false_type
{
};
template <typename T> struct is_complex<std::complex<T>> : std::true_type
{
};
template <typename T>
inline constexpr bool is_execution_policy_v = std::is_execution_policy_v<std::remove_cvref_t<T>>;
template <typename T>
concept execution_policy = is_execution_policy_v<T>;

// Minimal row-major view (the library's own mdspan stand-in).
template <typename T, size_t R> struct Span
{
    T *ptr = nullptr;
    std::array<size_t, R> ext{};
    Span() = default;
    template <typename... I>
    explicit Span(T *p, I... e) : ptr(p), ext{static_cast<size_t>(e)...}
    {
        static_assert(sizeof...(I) == R, "extent count must match the rank");
    }
    static constexpr size_t rank()
    {
        return R;
    }
    T *data_handle() const
    {
        return ptr;
    }
    size_t extent(size_t r) const
    {
        return ext[r];
    }
    size_t size() const
    {
        size_t s = 1;
        for (size_t e : ext)
            s *= e;
        return s;
    }
    template <typename... I> T &operator()(I... i) const
    {
        static_assert(sizeof...(I) == R);
        const size_t idx[] = {static_cast<size_t>(i)...};
        size_t off = 0;
        for (size_t r = 0; r < R; ++r)
            off = off * ext[r] + idx[r];
        return ptr[off];
    }
    T &operator[](size_t i) const
    {
        return ptr[i];
    }
};

namespace detail
{

// Map a libfpg status to the reference's exception types.
inline void check(int rc)
{
    if (rc == FPG_OK)
        return;
    const std::string msg = fpg_last_error();
    if (rc == FPG_ERR_INVALID)
        throw std::invalid_argument(msg);
    throw std::runtime_error("fast_pauli (GPU): " + msg);
}

inline void cuda_check(cudaError_t e, const char *where)
{
    if (e != cudaSuccess)
        throw std::runtime_error(std::string("fast_pauli (GPU): ") + where + ": " + cudaGetErrorString(e));
}

template <typename V> using elem_t = std::remove_cv_t<std::remove_pointer_t<decltype(std::declval<V>().data_handle())>>;

template <typename C> constexpr int32_t dtype_of()
{
    if constexpr (std::is_same_v<C, std::complex<double>>)
        return FPG_C128;
    else
    {
        static_assert(std::is_same_v<C, std::complex<float>>, "complex<double> or complex<float> arrays only");
        return FPG_C64;
    }
}

inline bool on_device(const void *p)
{
    int d = 0;
    check(fpg_pointer_is_device(p, &d));
    return d != 0;
}

// Stream-ordered device buffer from the library's pool (fpg_device_alloc),
// freed stream-ordered on scope exit, so temporaries never force a
// device-wide synchronisation and stay mapped for the next call.
struct DevBuf
{
    void *p = nullptr;
    size_t bytes = 0;
    cudaStream_t st = nullptr;
    DevBuf() = default;
    DevBuf(size_t n, cudaStream_t s) : bytes(n), st(s)
    {
        if (n)
            check(fpg_device_alloc(&p, n, s));
    }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), bytes(o.bytes), st(o.st)
    {
        o.p = nullptr;
    }
    ~DevBuf()
    {
        if (p)
            fpg_device_free(p, st);
    }
};

inline bool pinned_host(const void *p);

// A zero-valued host output written on the host (its pages made resident)
// before the device copies the result into it; page-locked memory is resident
// already.
inline void touch_host_output(void *p, size_t bytes)
{
    if (bytes && !pinned_host(p))
        std::memset(p, 0, bytes);
}

// A host or device array made available on the device for one call.
// mode: 0 = input (copied in), 1 = accumulating output (copied in and out),
// 2 = output known to be zero (memset, copied out).
class Staged
{
  public:
    Staged(const void *host_or_dev, size_t bytes, int mode, cudaStream_t st)
        : src_(const_cast<void *>(host_or_dev)), bytes_(bytes), mode_(mode), st_(st)
    {
        if (bytes == 0 || on_device(host_or_dev))
        {
            dev_ = src_;
            return;
        }
        buf_ = std::make_unique<DevBuf>(bytes, st);
        dev_ = buf_->p;
        if (mode == 2)
            cuda_check(cudaMemsetAsync(dev_, 0, bytes, st), "cudaMemsetAsync");
        else
            cuda_check(cudaMemcpyAsync(dev_, src_, bytes, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    }
    void *dev() const
    {
        return dev_;
    }
    bool staged() const
    {
        return buf_ != nullptr;
    }
    // Called once the call's device work is queued.  A zero output in
    // pageable memory is written on the host first (the values do not change)
    // while the device computes: a freshly allocated result (numpy.zeros'
    // untouched pages) otherwise takes its page faults inside the
    // device-to-host copy, on the GB300's Grace host several times slower.
    void finish()
    {
        if (buf_ && mode_ == 2)
            touch_host_output(src_, bytes_);
        if (buf_ && mode_ != 0)
            cuda_check(cudaMemcpyAsync(src_, dev_, bytes_, cudaMemcpyDeviceToHost, st_), "cudaMemcpyAsync");
    }

  private:
    void *src_;
    size_t bytes_;
    int mode_;
    cudaStream_t st_;
    void *dev_ = nullptr;
    std::unique_ptr<DevBuf> buf_;
};

// Stream of the calling thread: cudaStreamPerThread unless a caller (e.g. the
// Python bindings, for torch tensors) installs its own with StreamScope.
struct StreamChoice
{
    bool set = false;
    cudaStream_t s = nullptr; // may legitimately be the legacy default stream (0)
};
inline StreamChoice &stream_override()
{
    static thread_local StreamChoice c;
    return c;
}
inline cudaStream_t stream()
{
    const StreamChoice &c = stream_override();
    return c.set ? c.s : cudaStreamPerThread;
}
struct StreamScope
{
    StreamChoice prev;
    explicit StreamScope(cudaStream_t s) : prev(stream_override())
    {
        stream_override() = StreamChoice{true, s};
    }
    ~StreamScope()
    {
        stream_override() = prev;
    }
};

inline void sync(cudaStream_t st)
{
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
}

// Page-locked host memory (cudaHostAlloc / cudaHostRegister): copies from it
// are asynchronous, so they can overlap computation.
inline bool pinned_host(const void *p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// The calling thread's stream for host-to-device copies that overlap the
// computation on the call's stream (created on first use).
inline cudaStream_t copy_stream()
{
    struct Holder
    {
        cudaStream_t s = nullptr;
        ~Holder()
        {
            if (s)
                cudaStreamDestroy(s);
        }
    };
    static thread_local Holder h;
    if (!h.s)
        cuda_check(cudaStreamCreateWithFlags(&h.s, cudaStreamNonBlocking), "cudaStreamCreateWithFlags");
    return h.s;
}

// A second compute stream per host thread, for work that may run beside the
// call's stream (column chunks of one call).
inline cudaStream_t second_stream()
{
    struct Holder
    {
        cudaStream_t s = nullptr;
        ~Holder()
        {
            if (s)
                cudaStreamDestroy(s);
        }
    };
    static thread_local Holder h;
    if (!h.s)
        cuda_check(cudaStreamCreateWithFlags(&h.s, cudaStreamNonBlocking), "cudaStreamCreateWithFlags");
    return h.s;
}

struct Event
{
    cudaEvent_t e = nullptr;
    Event()
    {
        cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreateWithFlags");
    }
    Event(const Event &) = delete;
    Event &operator=(const Event &) = delete;
    ~Event()
    {
        cudaEventDestroy(e);
    }
};

// Column chunks of a call whose states are `bytes` of host memory in S
// columns: chunk c + 1 is copied in while chunk c is computed (columns are
// independent).  A narrower call costs more per column, so few chunks: three
// from 256 MiB and 512 columns, two from 64 MiB and 256 columns, else one
// (no overlap); the environment variable FPG_HOST_CHUNKS overrides the count.
inline size_t host_column_chunks(size_t S, size_t bytes)
{
    const size_t most = std::max<size_t>(1, S / 64);
    if (const char *e = std::getenv("FPG_HOST_CHUNKS"))
    {
        const long v = std::strtol(e, nullptr, 10);
        if (v >= 1)
            return std::min<size_t>((size_t)v, most);
    }
    if (bytes < (size_t(64) << 20) || S < 256)
        return 1;
    if (bytes >= (size_t(256) << 20) && S >= 512)
        return std::min<size_t>(3, most);
    return std::min<size_t>(2, most);
}

// Host-visible results must be complete before returning; device-resident
// calls stay asynchronous (stream ordered), like any CUDA library call.
inline void finish_call(cudaStream_t st, std::initializer_list<const Staged *> arrays)
{
    for (const Staged *a : arrays)
        if (a->staged())
        {
            sync(st);
            return;
        }
}

// Encoded strings cached per object, rebuilt when the strings change.
struct OpHandle
{
    fpg_operator *op = nullptr;
    explicit OpHandle(fpg_operator *o) : op(o)
    {
    }
    ~OpHandle()
    {
        if (op)
            fpg_operator_destroy(op);
    }
};

} // namespace detail

// Return the library pool's unused device memory (temporaries of earlier
// calls, kept mapped for reuse) to the device.
inline void release_cached_memory()
{
    detail::check(fpg_release_cached_memory());
}

// ---------------------------------------------------------------------------
// Pauli (reference: __pauli.hpp:39-212)
// ---------------------------------------------------------------------------
struct Pauli
{
    uint8_t code; // 0: I, 1: X, 2: Y, 3: Z

    constexpr Pauli() : code(0)
    {
    }
    template <class T>
        requires(std::is_integral_v<T> && !std::is_same_v<T, char>)
    constexpr Pauli(T const c) : code(static_cast<uint8_t>(c))
    {
        if (c < 0 || c > 3)
            throw std::invalid_argument("Pauli code must be 0, 1, 2, or 3");
    }
    constexpr Pauli(char const symbol) : code(0)
    {
        switch (symbol)
        {
        case 'I': code = 0; break;
        case 'X': code = 1; break;
        case 'Y': code = 2; break;
        case 'Z': code = 3; break;
        default: throw std::invalid_argument("Invalid Pauli matrix symbol");
        }
    }
    Pauli(Pauli const &) = default;
    Pauli &operator=(Pauli const &) noexcept = default;
    friend auto operator<=>(Pauli const &, Pauli const &) = default;

    char symbol() const
    {
        return "IXYZ"[code & 3];
    }

    // Product table with phases (reference: __pauli.hpp:110-178), computed
    // from the symplectic form: P_a P_b = i^{eps(a,b)} P_{a^b} with
    // eps = +1 for the cyclic order X->Y->Z, -1 for the anti-cyclic order.
    friend std::pair<std::complex<double>, Pauli> operator*(Pauli const &lhs, Pauli const &rhs)
    {
        const int a = lhs.code, b = rhs.code;
        if (a > 3 || b > 3)
            throw std::runtime_error("Unexpected Pauli code");
        Pauli r;
        r.code = static_cast<uint8_t>(a ^ b);
        if (a == 0 || b == 0 || a == b)
            return {1.0, r};
        // cyclic successor: X(1)->Y(2)->Z(3)->X(1)
        const int next = a % 3 + 1;
        return {next == b ? std::complex<double>(0, 1) : std::complex<double>(0, -1), r};
    }

    template <typename View> void to_tensor(View output) const
    {
        if (output.extent(0) != 2 || output.extent(1) != 2)
            throw std::invalid_argument("Output tensor must have (2, 2) shape");
        using C = detail::elem_t<View>;
        C *o = output.data_handle();
        const C I(0, 1);
        switch (code)
        {
        case 0: o[0] = 1; o[1] = 0; o[2] = 0; o[3] = 1; break;
        case 1: o[0] = 0; o[1] = 1; o[2] = 1; o[3] = 0; break;
        case 2: o[0] = 0; o[1] = -I; o[2] = I; o[3] = 0; break;
        case 3: o[0] = 1; o[1] = 0; o[2] = 0; o[3] = -1; break;
        default: throw std::runtime_error("Unexpected Pauli code");
        }
    }
};

// ---------------------------------------------------------------------------
// PauliString (reference: __pauli_string.hpp:126-561)
// ---------------------------------------------------------------------------

template <std::floating_point T>
std::tuple<std::vector<size_t>, std::vector<std::complex<T>>> get_sparse_repr(std::vector<Pauli> const &paulis);

struct PauliString
{
    uint8_t weight = 0;
    std::vector<Pauli> paulis;

    PauliString() noexcept = default;
    PauliString(std::vector<Pauli> p) : weight(0), paulis(std::move(p))
    {
        for (auto const &q : paulis)
            weight += q.code > 0;
    }
    PauliString(std::string const &str) : weight(0)
    {
        paulis.reserve(str.size());
        for (char c : str)
        {
            switch (c)
            {
            case 'I': paulis.push_back(Pauli{0}); break;
            case 'X': paulis.push_back(Pauli{1}); ++weight; break;
            case 'Y': paulis.push_back(Pauli{2}); ++weight; break;
            case 'Z': paulis.push_back(Pauli{3}); ++weight; break;
            default: throw std::invalid_argument(std::string("Invalid Pauli character ") + c);
            }
        }
    }
    PauliString(char const *str) : PauliString(std::string(str))
    {
    }
    PauliString(PauliString const &) = default;
    PauliString(PauliString &&) noexcept = default;
    PauliString &operator=(PauliString const &) = default;
    PauliString &operator=(PauliString &&) noexcept = default;
    friend auto operator<=>(PauliString const &, PauliString const &) = default;

    size_t n_qubits() const noexcept
    {
        return paulis.size();
    }
    size_t dim() const noexcept
    {
        return paulis.size() ? size_t(1) << paulis.size() : 0;
    }
    std::string str() const
    {
        std::string s(paulis.size(), 'I');
        for (size_t i = 0; i < paulis.size(); ++i)
            s[i] = paulis[i].symbol();
        return s;
    }

    friend std::pair<std::complex<double>, PauliString> operator*(PauliString const &lhs, PauliString const &rhs)
    {
        if (lhs.dim() != rhs.dim())
            throw std::invalid_argument("PauliStrings must have the same size");
        std::complex<double> phase = 1;
        std::vector<Pauli> out;
        out.reserve(lhs.n_qubits());
        for (size_t i = 0; i < lhs.n_qubits(); ++i)
        {
            auto [p, q] = lhs.paulis[i] * rhs.paulis[i];
            phase *= p;
            out.push_back(q);
        }
        return {phase, PauliString(std::move(out))};
    }

    // --- GPU methods -------------------------------------------------------

    // 1-D apply: new_states += c * P states   (reference :297-341)
    template <typename OutV, typename InV>
    void apply(OutV new_states, InV states, detail::elem_t<InV> const c = detail::elem_t<InV>(1)) const
    {
        apply(std::execution::seq, new_states, states, c);
    }
    template <execution_policy EP, typename OutV, typename InV>
    void apply(EP &&, OutV new_states, InV states, detail::elem_t<InV> const c = detail::elem_t<InV>(1)) const
    {
        if (states.size() != dim())
            throw std::invalid_argument("Input vector size must match the number of qubits");
        if (states.size() != new_states.size())
            throw std::invalid_argument("new_states must have the same dimensions as states");
        run_apply(new_states.data_handle(), states.data_handle(), 1, c, false);
    }

    // batched apply on (dim, n_states) (reference :378-436)
    template <typename OutV, typename InV>
    void apply_batch(OutV new_states_T, InV const states_T, detail::elem_t<InV> const c) const
    {
        apply_batch(std::execution::seq, new_states_T, states_T, c);
    }
    template <execution_policy EP, typename OutV, typename InV>
    void apply_batch(EP &&, OutV new_states_T, InV const states_T, detail::elem_t<InV> const c) const
    {
        if (states_T.extent(0) != dim())
            throw std::invalid_argument("[PauliString] states shape (" + std::to_string(states_T.extent(0)) +
                                        ") must match the dimension of the operators (" + std::to_string(dim()) +
                                        ")");
        if (states_T.extent(0) != new_states_T.extent(0) || states_T.extent(1) != new_states_T.extent(1))
            throw std::invalid_argument("[PauliString] new_states must have the same dimensions as states");
        run_apply(new_states_T.data_handle(), states_T.data_handle(), states_T.extent(1), c, false);
    }

    // expectation values on (dim, n_states), accumulated (reference :471-538)
    template <typename OutV, typename InV>
    void expectation_value(OutV expectation_vals_out, InV states,
                           detail::elem_t<InV> const c = detail::elem_t<InV>(1)) const
    {
        expectation_value(std::execution::seq, expectation_vals_out, states, c);
    }
    template <execution_policy EP, typename OutV, typename InV>
    void expectation_value(EP &&, OutV expectation_vals_out, InV states,
                           detail::elem_t<InV> const c = detail::elem_t<InV>(1)) const
    {
        if (states.extent(0) != dim())
            throw std::invalid_argument("[PauliString] states shape (" + std::to_string(states.extent(0)) +
                                        ") must match the dimension of the operators (" + std::to_string(dim()) +
                                        ")");
        if (expectation_vals_out.extent(0) != states.extent(1))
            throw std::invalid_argument("[PauliString] expectation_vals_out shape must match the number of states");
        run_expect(expectation_vals_out.data_handle(), states.data_handle(), states.extent(1), c, false);
    }

    template <typename View> void to_tensor(View output) const
    {
        if (output.extent(0) != dim() || output.extent(1) != dim())
            throw std::invalid_argument("Output tensor must have the same dimensions as the PauliString");
        using C = detail::elem_t<View>;
        auto [k, m] = get_sparse_repr<typename C::value_type>(paulis);
        C *o = output.data_handle();
        for (size_t i = 0; i < k.size(); ++i)
            o[i * dim() + k[i]] = m[i];
    }

    // Internal entry points used by the bindings: out_zero = output is known
    // to be zero on entry (no upload of it).
    template <typename C>
    void run_apply(C *out, const C *psi, size_t S, C c, bool out_zero) const
    {
        if (dim() == 0 || S == 0)
            return;
        const std::string s = str();
        fpg_operator *op = nullptr;
        detail::check(fpg_operator_create(s.data(), 1, (int32_t)n_qubits(), &op));
        detail::OpHandle h(op);
        cudaStream_t st = detail::stream();
        const size_t bytes = dim() * S * sizeof(C);
        detail::Staged in(psi, bytes, 0, st), o(out, bytes, out_zero ? 2 : 1, st);
        detail::DevBuf dc(sizeof(C), st);
        detail::cuda_check(cudaMemcpyAsync(dc.p, &c, sizeof(C), cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        detail::check(fpg_apply(op, dc.p, in.dev(), o.dev(), (int64_t)S, detail::dtype_of<C>(), st));
        o.finish();
        detail::finish_call(st, {&in, &o});
    }

    template <typename C>
    void run_expect(C *ev_out, const C *psi, size_t S, C c, bool out_zero) const
    {
        if (dim() == 0 || S == 0)
            return;
        const std::string s = str();
        fpg_operator *op = nullptr;
        detail::check(fpg_operator_create(s.data(), 1, (int32_t)n_qubits(), &op));
        detail::OpHandle h(op);
        cudaStream_t st = detail::stream();
        detail::Staged in(psi, dim() * S * sizeof(C), 0, st), o(ev_out, S * sizeof(C), out_zero ? 2 : 1, st);
        detail::DevBuf dc(sizeof(C), st);
        detail::cuda_check(cudaMemcpyAsync(dc.p, &c, sizeof(C), cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        detail::check(fpg_summed_expect(op, dc.p, 1, in.dev(), o.dev(), (int64_t)S, detail::dtype_of<C>(), st));
        o.finish();
        detail::finish_call(st, {&in, &o});
    }
};

// ---------------------------------------------------------------------------
// get_sparse_repr (reference: __pauli_string.hpp:49-118), on the device
// ---------------------------------------------------------------------------
template <std::floating_point T>
std::tuple<std::vector<size_t>, std::vector<std::complex<T>>> get_sparse_repr(std::vector<Pauli> const &paulis)
{
    const size_t n = paulis.size();
    if (n == 0)
        return {};
    const size_t D = size_t(1) << n;
    std::string s(n, 'I');
    for (size_t i = 0; i < n; ++i)
        s[i] = paulis[i].symbol();
    cudaStream_t st = detail::stream();
    detail::DevBuf dk(D * sizeof(uint64_t), st), dm(D * sizeof(std::complex<double>), st);
    detail::check(fpg_sparse_repr(s.data(), (int32_t)n, (uint64_t *)dk.p, dm.p, st));
    std::vector<uint64_t> k64(D);
    std::vector<std::complex<double>> m64(D);
    detail::cuda_check(cudaMemcpyAsync(k64.data(), dk.p, D * sizeof(uint64_t), cudaMemcpyDeviceToHost, st),
                       "cudaMemcpyAsync");
    detail::cuda_check(
        cudaMemcpyAsync(m64.data(), dm.p, D * sizeof(std::complex<double>), cudaMemcpyDeviceToHost, st),
        "cudaMemcpyAsync");
    detail::sync(st);
    std::vector<size_t> k(k64.begin(), k64.end());
    std::vector<std::complex<T>> m(m64.begin(), m64.end());
    return {std::move(k), std::move(m)};
}

} // namespace fast_pauli

template <> struct std::hash<fast_pauli::PauliString>
{
    std::size_t operator()(fast_pauli::PauliString const &key) const
    {
        // FNV-1a over the codes; the reference hashes the formatted string
        // (__pauli_string.hpp:586-594), any consistent hash serves.
        uint64_t h = 1469598103934665603ull;
        for (auto const &p : key.paulis)
        {
            h ^= p.code;
            h *= 1099511628211ull;
        }
        h ^= key.paulis.size();
        return (std::size_t)h;
    }
};

namespace fast_pauli
{

// ---------------------------------------------------------------------------
// helpers (reference: __pauli_helpers.hpp:36-153)
// ---------------------------------------------------------------------------
inline std::vector<std::string> get_nontrivial_paulis(size_t const weight)
{
    if (weight == 0)
        return {};
    std::vector<std::string> set{"X", "Y", "Z"};
    for (size_t i = 1; i < weight; ++i)
    {
        std::vector<std::string> next;
        next.reserve(set.size() * 3);
        for (auto const &s : set)
            for (const char *p : {"X", "Y", "Z"})
                next.push_back(s + p);
        set = std::move(next);
    }
    return set;
}

// k-subsets of {0..n-1} in lexicographic order
inline std::vector<std::vector<size_t>> idx_combinations(size_t const n, size_t const k)
{
    std::vector<std::vector<size_t>> result;
    if (k > n)
        return result;
    std::vector<size_t> c(k);
    std::iota(c.begin(), c.end(), size_t(0));
    while (true)
    {
        result.push_back(c);
        // advance to the next combination
        size_t i = k;
        while (i > 0 && c[i - 1] == n - k + (i - 1))
            --i;
        if (i == 0)
            break;
        ++c[i - 1];
        for (size_t j = i; j < k; ++j)
            c[j] = c[j - 1] + 1;
    }
    return result;
}

inline std::vector<PauliString> calculate_pauli_strings(size_t const n_qubits, size_t const weight)
{
    if (weight == 0)
        return {PauliString(std::string(n_qubits, 'I'))};
    const std::string base(n_qubits, 'I');
    auto words = get_nontrivial_paulis(weight);
    auto combos = idx_combinations(n_qubits, weight);
    std::vector<PauliString> result;
    result.reserve(words.size() * combos.size());
    for (auto const &w : words)
        for (auto const &cmb : combos)
        {
            std::string s = base;
            for (size_t q = 0; q < cmb.size(); ++q)
                s[cmb[q]] = w[q];
            result.emplace_back(s);
        }
    return result;
}

inline std::vector<PauliString> calculate_pauli_strings_max_weight(size_t n_qubits, size_t weight)
{
    std::vector<PauliString> result;
    for (size_t w = 0; w <= weight; ++w)
    {
        auto ps = calculate_pauli_strings(n_qubits, w);
        result.insert(result.end(), ps.begin(), ps.end());
    }
    return result;
}

namespace detail
{

inline std::string join_strings(std::vector<PauliString> const &ps)
{
    std::string s;
    if (ps.empty())
        return s;
    s.reserve(ps.size() * ps[0].n_qubits());
    for (auto const &p : ps)
        for (auto const &q : p.paulis)
            s.push_back(q.symbol());
    return s;
}

// Encoded-operator cache keyed by the strings' content.
// PauliString of the (x, z) masks (bit n-1-q is character q)
inline PauliString string_from_masks(uint64_t x, uint64_t z, size_t n)
{
    std::vector<Pauli> ps;
    ps.reserve(n);
    for (size_t q = 0; q < n; ++q)
    {
        const int b = (int)(n - 1 - q);
        const bool xb = (x >> b) & 1ull, zb = (z >> b) & 1ull;
        ps.push_back(Pauli(xb ? (zb ? 'Y' : 'X') : (zb ? 'Z' : 'I')));
    }
    return PauliString(std::move(ps));
}

class EncodedCache
{
  public:
    fpg_operator *get(std::vector<PauliString> const &ps) const
    {
        const std::string joined = join_strings(ps);
        std::lock_guard<std::mutex> lk(mu_);
        if (h_ && key_ == joined)
            return h_->op;
        fpg_operator *op = nullptr;
        check(fpg_operator_create(joined.data(), (int64_t)ps.size(), (int32_t)ps[0].n_qubits(), &op));
        h_ = std::make_shared<OpHandle>(op);
        key_ = joined;
        return op;
    }

  private:
    mutable std::mutex mu_;
    mutable std::shared_ptr<OpHandle> h_;
    mutable std::string key_;
};

} // namespace detail

// ---------------------------------------------------------------------------
// PauliOp (reference: __pauli_op.hpp:38-592)
// ---------------------------------------------------------------------------
template <std::floating_point T, typename H = std::complex<T>> struct PauliOp
{
    std::vector<H> coeffs;
    std::vector<PauliString> pauli_strings;

    PauliOp() = default;
    PauliOp(std::vector<std::string> const &strings)
    {
        for (auto const &s : strings)
            pauli_strings.push_back(PauliString(s));
        coeffs.resize(pauli_strings.size(), H(1.0));
        validate_pauli_strings(pauli_strings);
    }
    PauliOp(std::vector<PauliString> strings) : coeffs(strings.size(), H(1.0)), pauli_strings(std::move(strings))
    {
        validate_pauli_strings(pauli_strings);
    }
    PauliOp(std::vector<H> coefficients, std::vector<PauliString> strings)
        : coeffs(std::move(coefficients)), pauli_strings(std::move(strings))
    {
        if (coeffs.size() != pauli_strings.size())
            throw std::invalid_argument("coeffs and pauli_strings must have the same size");
        validate_pauli_strings(pauli_strings);
    }
    PauliOp(PauliOp const &o) : coeffs(o.coeffs), pauli_strings(o.pauli_strings)
    {
    }
    PauliOp(PauliOp &&o) noexcept : coeffs(std::move(o.coeffs)), pauli_strings(std::move(o.pauli_strings))
    {
    }
    PauliOp &operator=(PauliOp const &o)
    {
        coeffs = o.coeffs;
        pauli_strings = o.pauli_strings;
        return *this;
    }
    PauliOp &operator=(PauliOp &&o) noexcept
    {
        coeffs = std::move(o.coeffs);
        pauli_strings = std::move(o.pauli_strings);
        return *this;
    }

    size_t dim() const
    {
        return pauli_strings.empty() ? 0 : pauli_strings[0].dim();
    }
    size_t n_qubits() const
    {
        return pauli_strings.empty() ? 0 : pauli_strings[0].n_qubits();
    }
    size_t n_pauli_strings() const
    {
        return pauli_strings.size();
    }

    void scale(std::complex<T> factor)
    {
        for (auto &c : coeffs)
            c *= factor;
    }
    template <typename View>
        requires requires(View v) { v.data_handle(); }
    void scale(View factors)
    {
        if (factors.size() != n_pauli_strings())
            throw std::invalid_argument("factors must have the same length as the number of PauliStrings");
        for (size_t i = 0; i < coeffs.size(); ++i)
            coeffs[i] *= factors.data_handle()[i];
    }

    PauliOp operator-() const
    {
        std::vector<H> neg(coeffs.size());
        std::transform(coeffs.begin(), coeffs.end(), neg.begin(), [](H const &c) { return -c; });
        return PauliOp(std::move(neg), pauli_strings);
    }

    friend PauliOp operator*(PauliOp const &lhs, PauliString const &rhs)
    {
        if (lhs.dim() != rhs.dim())
            throw std::invalid_argument("PauliStrings must have same size as PauliOp");
        std::vector<H> c(lhs.coeffs);
        std::vector<PauliString> s;
        s.reserve(lhs.n_pauli_strings());
        for (size_t i = 0; i < lhs.n_pauli_strings(); ++i)
        {
            auto [ph, p] = lhs.pauli_strings[i] * rhs;
            c[i] *= H(ph);
            s.push_back(std::move(p));
        }
        return PauliOp(std::move(c), std::move(s));
    }
    friend PauliOp operator*(PauliString const &lhs, PauliOp const &rhs)
    {
        if (lhs.dim() != rhs.dim())
            throw std::invalid_argument("PauliStrings must have same size as PauliOp");
        std::vector<H> c(rhs.coeffs);
        std::vector<PauliString> s;
        s.reserve(rhs.n_pauli_strings());
        for (size_t i = 0; i < rhs.n_pauli_strings(); ++i)
        {
            auto [ph, p] = lhs * rhs.pauli_strings[i];
            c[i] *= H(ph);
            s.push_back(std::move(p));
        }
        return PauliOp(std::move(c), std::move(s));
    }
    // Product of two operators with equal strings merged (reference
    // :237-281), on the GPU (fpg_op_product): the distinct product strings
    // ordered by their (x, z) encoding, coefficients summed in pair order.
    // (The reference's order is that of its per-thread hash maps.)
    friend PauliOp operator*(PauliOp const &lhs, PauliOp const &rhs)
    {
        if (lhs.dim() != rhs.dim())
            throw std::invalid_argument("Mismatched dimensions for provided PauliOp");
        const size_t Pa = lhs.n_pauli_strings(), Pb = rhs.n_pauli_strings();
        if (Pa == 0 || Pb == 0)
            return PauliOp();
        const size_t n = lhs.pauli_strings[0].n_qubits();
        using CD = std::complex<double>;
        if (n == 0)
        {
            // strings without characters: scalars
            CD sa = 0, sb = 0;
            for (auto const &c : lhs.coeffs)
                sa += CD(c);
            for (auto const &c : rhs.coeffs)
                sb += CD(c);
            return PauliOp(std::vector<H>{H(sa * sb)}, std::vector<PauliString>{PauliString(std::vector<Pauli>{})});
        }
        const size_t N = Pa * Pb;
        if (N >= (size_t(1) << 31))
            throw std::runtime_error("fast_pauli (GPU): too many string pairs in a PauliOp product (>= 2^31)");
        fpg_operator *oa = lhs.cache_.get(lhs.pauli_strings), *ob = rhs.cache_.get(rhs.pauli_strings);
        cudaStream_t st = detail::stream();
        const std::vector<CD> ca(lhs.coeffs.begin(), lhs.coeffs.end()), cb(rhs.coeffs.begin(), rhs.coeffs.end());
        detail::DevBuf da(Pa * sizeof(CD), st), db(Pb * sizeof(CD), st), ox(N * 8, st), oz(N * 8, st),
            oc(N * sizeof(CD), st);
        detail::cuda_check(cudaMemcpyAsync(da.p, ca.data(), da.bytes, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        detail::cuda_check(cudaMemcpyAsync(db.p, cb.data(), db.bytes, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        int64_t n_out = 0;
        detail::check(fpg_op_product(oa, da.p, ob, db.p, (uint64_t *)ox.p, (uint64_t *)oz.p, oc.p, &n_out, st));
        std::vector<uint64_t> hx((size_t)n_out), hz((size_t)n_out);
        std::vector<CD> hc((size_t)n_out);
        if (n_out > 0)
        {
            detail::cuda_check(cudaMemcpyAsync(hx.data(), ox.p, hx.size() * 8, cudaMemcpyDeviceToHost, st),
                               "cudaMemcpyAsync");
            detail::cuda_check(cudaMemcpyAsync(hz.data(), oz.p, hz.size() * 8, cudaMemcpyDeviceToHost, st),
                               "cudaMemcpyAsync");
            detail::cuda_check(cudaMemcpyAsync(hc.data(), oc.p, hc.size() * sizeof(CD), cudaMemcpyDeviceToHost, st),
                               "cudaMemcpyAsync");
        }
        detail::sync(st);
        std::vector<H> c;
        std::vector<PauliString> strs;
        c.reserve(hc.size());
        strs.reserve(hc.size());
        for (size_t k = 0; k < hc.size(); ++k)
        {
            c.push_back(H(hc[k]));
            strs.push_back(detail::string_from_masks(hx[k], hz[k], n));
        }
        return PauliOp(std::move(c), std::move(strs));
    }

    void extend(PauliString pauli_str, std::complex<T> coeff, bool dedupe = true)
    {
        if (pauli_str.dim() != dim())
            throw std::invalid_argument("PauliStrings must have same size as PauliOp");
        if (dedupe)
            for (size_t i = 0; i < pauli_strings.size(); ++i)
                if (pauli_strings[i] == pauli_str)
                {
                    coeffs[i] += coeff;
                    return;
                }
        coeffs.push_back(coeff);
        pauli_strings.push_back(std::move(pauli_str));
    }
    void extend(PauliOp const &other)
    {
        if (other.dim() != dim())
            throw std::invalid_argument("Mismatched dimensions for provided PauliOp");
        PauliOp copy(other); // other may alias *this
        pauli_strings.insert(pauli_strings.end(), copy.pauli_strings.begin(), copy.pauli_strings.end());
        coeffs.insert(coeffs.end(), copy.coeffs.begin(), copy.coeffs.end());
    }

    // --- GPU methods -------------------------------------------------------

    template <typename OutV, typename InV> void apply(OutV new_states, InV const states) const
    {
        apply(std::execution::seq, new_states, states);
    }
    template <execution_policy EP, typename OutV, typename InV> void apply(EP &&, OutV new_states, InV const states) const
    {
        const size_t S = states.rank() == 1 ? 1 : states.extent(1);
        const size_t Sn = new_states.rank() == 1 ? 1 : new_states.extent(1);
        if (states.extent(0) != dim())
            throw std::invalid_argument("[PauliOp] state size must match the dimension of the operators");
        if (states.extent(0) != new_states.extent(0) || S != Sn)
            throw std::invalid_argument("[PauliOp] new_states must have the same dimensions as states");
        run_apply(new_states.data_handle(), states.data_handle(), S, false);
    }

    template <typename OutV, typename InV> void expectation_value(OutV expectation_vals_out, InV states) const
    {
        expectation_value(std::execution::seq, expectation_vals_out, states);
    }
    template <execution_policy EP, typename OutV, typename InV>
    void expectation_value(EP &&, OutV expectation_vals_out, InV states) const
    {
        if (states.extent(0) != dim())
            throw std::invalid_argument("[PauliOp] state size must match the dimension of the operators");
        const size_t S = states.rank() == 1 ? 1 : states.extent(1);
        if (expectation_vals_out.extent(0) != S)
            throw std::invalid_argument("[PauliOp] expectation_vals_out shape must match the number of states");
        run_expect(expectation_vals_out.data_handle(), states.data_handle(), S, false);
    }

    // Dense matrix, accumulated into output (reference :558-571), on the GPU
    // (fpg_to_tensor).
    template <typename View> void to_tensor(View output) const
    {
        using C = detail::elem_t<View>;
        if (pauli_strings.empty() || dim() == 0)
            return;
        fpg_operator *op = cache_.get(pauli_strings);
        cudaStream_t st = detail::stream();
        detail::Staged o(output.data_handle(), dim() * dim() * sizeof(C), 1, st);
        std::vector<C> c(coeffs.begin(), coeffs.end());
        detail::DevBuf dc(c.size() * sizeof(C), st);
        detail::cuda_check(cudaMemcpyAsync(dc.p, c.data(), dc.bytes, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        detail::check(fpg_to_tensor(op, dc.p, 1, o.dev(), detail::dtype_of<C>(), st));
        o.finish();
        detail::finish_call(st, {&o});
    }

    static inline void validate_pauli_strings(std::vector<PauliString> const &ps)
    {
        if (!ps.empty())
        {
            const size_t n = ps[0].n_qubits();
            if (!std::all_of(ps.begin(), ps.end(), [n](PauliString const &p) { return p.n_qubits() == n; }))
                throw std::invalid_argument("All PauliStrings must have the same size");
        }
    }

    // Internal entry points used by the bindings.
    template <typename C> void run_apply(C *out, const C *psi, size_t S, bool out_zero) const
    {
        if (dim() == 0 || S == 0 || pauli_strings.empty())
            return;
        fpg_operator *op = cache_.get(pauli_strings);
        cudaStream_t st = detail::stream();
        const size_t bytes = dim() * S * sizeof(C);
        detail::Staged in(psi, bytes, 0, st), o(out, bytes, out_zero ? 2 : 1, st);
        std::vector<C> c(coeffs.begin(), coeffs.end());
        detail::DevBuf dc(c.size() * sizeof(C), st);
        detail::cuda_check(cudaMemcpyAsync(dc.p, c.data(), dc.bytes, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        detail::check(fpg_apply(op, dc.p, in.dev(), o.dev(), (int64_t)S, detail::dtype_of<C>(), st));
        o.finish();
        detail::finish_call(st, {&in, &o});
    }
    template <typename C> void run_expect(C *ev_out, const C *psi, size_t S, bool out_zero) const
    {
        if (dim() == 0 || S == 0 || pauli_strings.empty())
            return;
        fpg_operator *op = cache_.get(pauli_strings);
        cudaStream_t st = detail::stream();
        detail::Staged in(psi, dim() * S * sizeof(C), 0, st), o(ev_out, S * sizeof(C), out_zero ? 2 : 1, st);
        std::vector<C> c(coeffs.begin(), coeffs.end());
        detail::DevBuf dc(c.size() * sizeof(C), st);
        detail::cuda_check(cudaMemcpyAsync(dc.p, c.data(), dc.bytes, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        detail::check(fpg_summed_expect(op, dc.p, 1, in.dev(), o.dev(), (int64_t)S, detail::dtype_of<C>(), st));
        o.finish();
        detail::finish_call(st, {&in, &o});
    }

  private:
    detail::EncodedCache cache_;
};

// ---------------------------------------------------------------------------
// SummedPauliOp (reference: __summed_pauli_op.hpp:37-666)
// ---------------------------------------------------------------------------
template <std::floating_point T> struct SummedPauliOp
{
    template <size_t N> using Tensor = Span<std::complex<T>, N>;

    std::vector<PauliString> pauli_strings;
    std::vector<std::complex<T>> coeffs_raw;
    Tensor<2> coeffs; // (n_pauli_strings, n_operators), views coeffs_raw

    SummedPauliOp() noexcept = default;

    SummedPauliOp(std::vector<PauliString> const &ps, std::vector<std::complex<T>> const &raw)
        : pauli_strings(ps), coeffs_raw(raw)
    {
        const size_t P = pauli_strings.size();
        const size_t K = P ? coeffs_raw.size() / P : 0;
        coeffs = Tensor<2>(coeffs_raw.data(), P, K);
        check_ctor_inputs(pauli_strings, P);
    }
    template <typename View>
        requires requires(View v) { v.data_handle(); v.extent(1); }
    SummedPauliOp(std::vector<PauliString> const &ps, View const c) : pauli_strings(ps)
    {
        check_ctor_inputs(pauli_strings, c.extent(0));
        copy_coeffs(c);
    }
    template <typename View>
        requires requires(View v) { v.data_handle(); v.extent(1); }
    SummedPauliOp(std::vector<std::string> const &strs, View const c)
    {
        for (auto const &s : strs)
            pauli_strings.push_back(PauliString(s));
        check_ctor_inputs(pauli_strings, c.extent(0));
        copy_coeffs(c);
    }
    SummedPauliOp(SummedPauliOp const &o) : pauli_strings(o.pauli_strings), coeffs_raw(o.coeffs_raw)
    {
        coeffs = Tensor<2>(coeffs_raw.data(), o.coeffs.extent(0), o.coeffs.extent(1));
    }
    SummedPauliOp &operator=(SummedPauliOp const &o)
    {
        pauli_strings = o.pauli_strings;
        coeffs_raw = o.coeffs_raw;
        coeffs = Tensor<2>(coeffs_raw.data(), o.coeffs.extent(0), o.coeffs.extent(1));
        return *this;
    }

    size_t dim() const noexcept
    {
        return pauli_strings.empty() ? 0 : pauli_strings[0].dim();
    }
    size_t n_qubits() const noexcept
    {
        return pauli_strings.empty() ? 0 : pauli_strings[0].n_qubits();
    }
    size_t n_operators() const noexcept
    {
        return coeffs.extent(1);
    }
    size_t n_pauli_strings() const noexcept
    {
        return pauli_strings.size();
    }

    // --- GPU methods -------------------------------------------------------

    template <typename OutV, typename InV> void apply(OutV new_states, InV states) const
    {
        apply(std::execution::seq, new_states, states);
    }
    template <execution_policy EP, typename OutV, typename InV> void apply(EP &&, OutV new_states, InV states) const
    {
        if (states.extent(0) != new_states.extent(0) || states.extent(1) != new_states.extent(1))
            throw std::invalid_argument("new_states must have the same dimensions as states");
        if (states.extent(0) != dim())
            throw std::invalid_argument("state size must match the dimension of the operators");
        run_apply(new_states.data_handle(), states.data_handle(), states.extent(1), false);
    }

    template <typename OutV, typename InV, typename DataV>
    void apply_weighted(OutV new_states, InV states, DataV data) const
    {
        apply_weighted(std::execution::seq, new_states, states, data);
    }
    template <execution_policy EP, typename OutV, typename InV, typename DataV>
    void apply_weighted(EP &&, OutV new_states, InV states, DataV data) const
    {
        if (states.extent(0) != new_states.extent(0) || states.extent(1) != new_states.extent(1))
            throw std::invalid_argument("new_states must have the same dimensions as states");
        if (data.extent(0) != n_operators() || data.extent(1) != states.extent(1))
            throw std::invalid_argument("data(k,t) must have the same number of operators as the SummedPauliOp and "
                                        "the same number of states as the input states");
        if (states.extent(0) != dim())
            throw std::invalid_argument("state size must match the dimension of the operators");
        run_apply_weighted(new_states.data_handle(), states.data_handle(), data.data_handle(), states.extent(1),
                           false);
    }

    template <typename OutV, typename InV> void expectation_value(OutV expectation_vals_out, InV states) const
    {
        expectation_value(std::execution::seq, expectation_vals_out, states);
    }
    template <execution_policy EP, typename OutV, typename InV>
    void expectation_value(EP &&, OutV expectation_vals_out, InV states) const
    {
        const size_t S = states.extent(1), K = n_operators();
        if (expectation_vals_out.extent(0) != K)
            throw std::invalid_argument("expectation_vals_out must have the same number of operators (" +
                                        std::to_string(expectation_vals_out.extent(0)) +
                                        ") as the SummedPauliOp (" + std::to_string(K) + ")");
        if (states.extent(0) != dim())
            throw std::invalid_argument("states must have the same dimension (" + std::to_string(states.extent(0)) +
                                        ") as the SummedPauliOp (" + std::to_string(dim()) + ")");
        if (expectation_vals_out.extent(1) != S)
            throw std::invalid_argument("expectation_vals_out must have the same number of states (" +
                                        std::to_string(expectation_vals_out.extent(1)) +
                                        ") as the input states (" + std::to_string(S) + ")");
        run_expect(expectation_vals_out.data_handle(), states.data_handle(), S, false);
    }

    // Host-side (not on the GPU path): components as PauliOps (reference :621-637)
    std::vector<PauliOp<T>> split() const
    {
        std::vector<PauliOp<T>> ops;
        ops.reserve(n_operators());
        for (size_t k = 0; k < n_operators(); ++k)
        {
            std::vector<std::complex<T>> c(n_pauli_strings());
            for (size_t i = 0; i < n_pauli_strings(); ++i)
                c[i] = coeffs(i, k);
            ops.emplace_back(std::move(c), pauli_strings);
        }
        return ops;
    }

    // Square of each operator A_k -> A_k^2 (reference :197-268): the squared
    // string set as the reference (all strings of weight <= min(n, 2 w)),
    // coefficients from the GPU (fpg_summed_square).
    SummedPauliOp square() const
    {
        size_t weight = 0;
        for (auto const &p : pauli_strings)
            weight = std::max<size_t>(weight, p.weight);
        auto sq = calculate_pauli_strings_max_weight(n_qubits(), std::min(n_qubits(), 2 * weight));
        using C = std::complex<T>;
        const size_t K = n_operators(), A = sq.size();
        std::vector<C> out(A * K);
        if (!pauli_strings.empty() && K > 0 && A > 0)
        {
            fpg_operator *op = cache_.get(pauli_strings);
            const std::string joined = detail::join_strings(sq);
            fpg_operator *q = nullptr;
            detail::check(fpg_operator_create(joined.data(), (int64_t)A, (int32_t)n_qubits(), &q));
            detail::OpHandle qh(q);
            cudaStream_t st = detail::stream();
            detail::DevBuf dh = upload_coeffs<C>(st);
            detail::DevBuf dout(A * K * sizeof(C), st);
            detail::check(fpg_summed_square(op, dh.p, (int64_t)K, q, dout.p, detail::dtype_of<C>(), st));
            detail::cuda_check(cudaMemcpyAsync(out.data(), dout.p, dout.bytes, cudaMemcpyDeviceToHost, st),
                               "cudaMemcpyAsync");
            detail::sync(st);
        }
        return SummedPauliOp(sq, Tensor<2>(out.data(), A, K));
    }

    // Dense matrices (K, D, D), accumulated into A_k_out (reference :644-665),
    // on the GPU (fpg_to_tensor).
    template <typename View> void to_tensor(View A_k_out) const
    {
        using C = detail::elem_t<View>;
        const size_t D = dim(), K = n_operators();
        if (pauli_strings.empty() || D == 0 || K == 0)
            return;
        fpg_operator *op = cache_.get(pauli_strings);
        cudaStream_t st = detail::stream();
        detail::Staged o(A_k_out.data_handle(), K * D * D * sizeof(C), 1, st);
        detail::DevBuf dh = upload_coeffs<C>(st);
        detail::check(fpg_to_tensor(op, dh.p, (int64_t)K, o.dev(), detail::dtype_of<C>(), st));
        o.finish();
        detail::finish_call(st, {&o});
    }

    // Internal entry points used by the bindings.
    template <typename C> void run_apply(C *out, const C *psi, size_t S, bool out_zero) const
    {
        if (dim() == 0 || S == 0 || pauli_strings.empty())
            return;
        fpg_operator *op = cache_.get(pauli_strings);
        cudaStream_t st = detail::stream();
        const size_t bytes = dim() * S * sizeof(C);
        detail::Staged in(psi, bytes, 0, st), o(out, bytes, out_zero ? 2 : 1, st);
        detail::DevBuf dh = upload_coeffs<C>(st);
        detail::check(fpg_summed_apply(op, dh.p, (int64_t)n_operators(), in.dev(), o.dev(), (int64_t)S,
                                       detail::dtype_of<C>(), st));
        o.finish();
        detail::finish_call(st, {&in, &o});
    }
    template <typename C, typename R>
    void run_apply_weighted(C *out, const C *psi, const R *data, size_t S, bool out_zero) const
    {
        static_assert(std::is_same_v<R, typename C::value_type>, "data must be real of the states' precision");
        if (dim() == 0 || S == 0 || pauli_strings.empty())
            return;
        fpg_operator *op = cache_.get(pauli_strings);
        cudaStream_t st = detail::stream();
        const size_t bytes = dim() * S * sizeof(C);
        detail::Staged in(psi, bytes, 0, st), o(out, bytes, out_zero ? 2 : 1, st);
        detail::Staged dd(data, n_operators() * S * sizeof(R), 0, st);
        detail::DevBuf dh = upload_coeffs<C>(st);
        detail::check(fpg_summed_apply_weighted(op, dh.p, (int64_t)n_operators(), in.dev(), dd.dev(), o.dev(),
                                                (int64_t)S, detail::dtype_of<C>(), st));
        o.finish();
        detail::finish_call(st, {&in, &o, &dd});
    }
    template <typename C> void run_expect(C *out, const C *psi, size_t S, bool out_zero) const
    {
        if (dim() == 0 || S == 0 || pauli_strings.empty() || n_operators() == 0)
            return;
        fpg_operator *op = cache_.get(pauli_strings);
        cudaStream_t st = detail::stream();
        const size_t in_bytes = dim() * S * sizeof(C);
        if (!detail::on_device(out) && !detail::on_device(psi))
            if (const size_t nc = detail::host_column_chunks(S, in_bytes); nc > 1)
                return run_expect_overlapped(op, out, psi, S, out_zero, nc, st);
        detail::Staged in(psi, in_bytes, 0, st), o(out, n_operators() * S * sizeof(C), out_zero ? 2 : 1, st);
        detail::DevBuf dh = upload_coeffs<C>(st);
        detail::check(fpg_summed_expect(op, dh.p, (int64_t)n_operators(), in.dev(), o.dev(), (int64_t)S,
                                        detail::dtype_of<C>(), st));
        o.finish();
        detail::finish_call(st, {&in, &o});
    }

  private:
    detail::EncodedCache cache_;

    // Host states in nc column chunks: chunk c's copy goes on the thread's
    // copy stream (the link runs the copies back to back) and its computation
    // on a compute stream, ordered after that copy, before chunk c + 1's
    // copy is issued: from pinned memory the copies are asynchronous, and
    // from pageable memory, whose copies return only once the host has handed
    // the data over, chunk c is already running on the GPU while chunk
    // c + 1 is being copied.  The results are copied out after the last
    // chunk.  Each chunk is an independent fpg_summed_expect call on its own
    // columns; the chunks alternate between the call's stream and a second
    // compute stream, so that a chunk whose copy has landed starts while the
    // chunk before it runs its last, small kernels (reductions, the
    // contraction, whose GEMM fills few SMs at a chunk's width).
    template <typename C>
    void run_expect_overlapped(fpg_operator *op, C *out, const C *psi, size_t S, bool out_zero, size_t nc,
                               cudaStream_t st) const
    {
        const size_t D = dim(), K = n_operators(), el = sizeof(C);
        // widths in multiples of 64 columns: the first small, a quarter of S
        // with two chunks and an eighth with more (its copy is the part that
        // nothing hides; its computation then takes about as long as the
        // next chunk's copy), the rest split evenly, the remainder in the last
        // chunk.  n=14 weight<=2 workload, 1024 columns, pageable states:
        // 4.17 ms without chunks, 3.65 ms in two (a quarter first), 3.55 ms
        // in three (an eighth first); 3.72 / 3.75 ms for three / four with a
        // quarter first, 3.72 / 3.88 ms for four / five with an eighth
        std::vector<size_t> c0, cw;
        size_t left = S;
        const size_t first = nc > 2 ? S / 8 : S / 4;
        for (size_t c = 0; c < nc && left; ++c)
        {
            size_t w = c == 0 ? std::max<size_t>(64, first / 64 * 64)
                              : std::max<size_t>(64, left / (nc - c) / 64 * 64);
            w = c + 1 == nc ? left : std::min(w, left);
            c0.push_back(S - left);
            cw.push_back(w);
            left -= w;
        }
        cw.back() += left;
        nc = cw.size();
        detail::DevBuf dh = upload_coeffs<C>(st);
        std::vector<detail::DevBuf> din, dout;
        din.reserve(nc);
        dout.reserve(nc);
        for (size_t c = 0; c < nc; ++c)
        {
            din.emplace_back(D * cw[c] * el, st);
            dout.emplace_back(K * cw[c] * el, st);
        }
        cudaStream_t cs = detail::copy_stream();
        const cudaStream_t ss[2] = {st, detail::second_stream()};
        detail::Event fork, second_done;
        std::vector<std::unique_ptr<detail::Event>> landed(nc);
        // whatever happens below, the call's stream waits for every queued
        // copy and for the second compute stream before the buffers go back
        // to the pool on the call's stream
        struct JoinCopies
        {
            std::vector<std::unique_ptr<detail::Event>> &ev;
            cudaStream_t st, second;
            cudaEvent_t second_done;
            ~JoinCopies()
            {
                for (auto &e : ev)
                    if (e)
                        cudaStreamWaitEvent(st, e->e, 0);
                if (cudaEventRecord(second_done, second) == cudaSuccess)
                    cudaStreamWaitEvent(st, second_done, 0);
            }
        } join{landed, st, ss[1], second_done.e};
        detail::cuda_check(cudaEventRecord(fork.e, st), "cudaEventRecord");
        detail::cuda_check(cudaStreamWaitEvent(cs, fork.e, 0), "cudaStreamWaitEvent");
        detail::cuda_check(cudaStreamWaitEvent(ss[1], fork.e, 0), "cudaStreamWaitEvent");
        for (size_t c = 0; c < nc; ++c)
        {
            const cudaStream_t cst = ss[c & 1];
            detail::cuda_check(cudaMemcpy2DAsync(din[c].p, cw[c] * el, psi + c0[c], S * el, cw[c] * el, D,
                                                 cudaMemcpyHostToDevice, cs),
                               "cudaMemcpy2DAsync");
            // an accumulating output is copied in on the copy stream too: a
            // pageable copy on the call's stream would first wait for the
            // chunks already running there
            if (!out_zero)
                detail::cuda_check(cudaMemcpy2DAsync(dout[c].p, cw[c] * el, out + c0[c], S * el, cw[c] * el, K,
                                                     cudaMemcpyHostToDevice, cs),
                                   "cudaMemcpy2DAsync");
            landed[c] = std::make_unique<detail::Event>();
            detail::cuda_check(cudaEventRecord(landed[c]->e, cs), "cudaEventRecord");
            if (out_zero)
                detail::cuda_check(cudaMemsetAsync(dout[c].p, 0, dout[c].bytes, cst), "cudaMemsetAsync");
            detail::cuda_check(cudaStreamWaitEvent(cst, landed[c]->e, 0), "cudaStreamWaitEvent");
            detail::check(fpg_summed_expect(op, dh.p, (int64_t)K, din[c].p, dout[c].p, (int64_t)cw[c],
                                            detail::dtype_of<C>(), cst));
        }
        // a zero output: made resident on the host while the chunks run
        if (out_zero)
            detail::touch_host_output(out, K * S * el);
        detail::cuda_check(cudaEventRecord(second_done.e, ss[1]), "cudaEventRecord");
        detail::cuda_check(cudaStreamWaitEvent(st, second_done.e, 0), "cudaStreamWaitEvent");
        for (size_t c = 0; c < nc; ++c)
            detail::cuda_check(cudaMemcpy2DAsync(out + c0[c], S * el, dout[c].p, cw[c] * el, cw[c] * el, K,
                                                 cudaMemcpyDeviceToHost, st),
                               "cudaMemcpy2DAsync");
        detail::sync(st);
    }

    static void check_ctor_inputs(std::vector<PauliString> const &ps, size_t rows)
    {
        if (!ps.empty())
        {
            const size_t n = ps.front().n_qubits();
            if (!std::all_of(ps.begin(), ps.end(), [n](PauliString const &p) { return p.n_qubits() == n; }))
                throw std::invalid_argument("All PauliStrings must have the same size");
        }
        if (rows != ps.size())
            throw std::invalid_argument("The number of PauliStrings must match the number of rows in the coeffs "
                                        "matrix");
    }
    template <typename View> void copy_coeffs(View const c)
    {
        const size_t P = c.extent(0), K = c.extent(1);
        coeffs_raw.assign(c.data_handle(), c.data_handle() + P * K);
        coeffs = Tensor<2>(coeffs_raw.data(), P, K);
    }
    template <typename C> detail::DevBuf upload_coeffs(cudaStream_t st) const
    {
        detail::DevBuf d(coeffs_raw.size() * sizeof(C), st);
        if (!d.bytes)
            return d;
        if constexpr (std::is_same_v<C, std::complex<T>>)
        {
            // the stored coefficients as they are (a pageable-source copy
            // returns once the source has been staged)
            detail::cuda_check(cudaMemcpyAsync(d.p, coeffs_raw.data(), d.bytes, cudaMemcpyHostToDevice, st),
                               "cudaMemcpyAsync");
        }
        else
        {
            // converted first; the temporary may go out of scope once the
            // pageable-source copy has returned
            std::vector<C> c(coeffs_raw.begin(), coeffs_raw.end());
            detail::cuda_check(cudaMemcpyAsync(d.p, c.data(), d.bytes, cudaMemcpyHostToDevice, st),
                               "cudaMemcpyAsync");
        }
        return d;
    }
};

} // namespace fast_pauli
