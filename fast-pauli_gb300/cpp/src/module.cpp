// module.cpp -- Python module fast_pauli._fast_pauli over the C++ host API.
//
// Mirrors the reference's nanobind module (fast_pauli/cpp/src/fast_pauli.cpp:28-106
// and fast_pauli/cpp/src/include/__*_bindings.hpp): same classes, methods,
// properties, keyword names, return shapes, pickle tuples and ValueError
// contract.  Built with pybind11 (the copy bundled with torch); nanobind is
// not available offline.
//
// Arrays:
//  * numpy (or anything numpy.asarray accepts): complex128 arrays must be
//    C-contiguous (else ValueError, reference __nb_helpers.hpp:55-74); other
//    dtypes are converted to a contiguous complex128 copy (nanobind's implicit
//    conversion).  Computed in float64 on the GPU; results are new numpy arrays.
//  * CUDA tensors (objects exposing __cuda_array_interface__, e.g. torch):
//    used in place, no host copies, ordered on torch's current stream;
//    complex128 -> float64 path, complex64 -> mixed float32 path.  Results are
//    new tensors of the input's type and device.
// The GIL is released around GPU work.
#include <pybind11/complex.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <sstream>

#include "fast_pauli_gb300.hpp"

namespace py = pybind11;
namespace fp = fast_pauli;
using namespace pybind11::literals;

using cd = std::complex<double>;
using cf = std::complex<float>;

namespace
{

// ---------------------------------------------------------------------------
// array marshalling
// ---------------------------------------------------------------------------

enum class Kind
{
    C128,
    C64,
    F64,
    F32
};

struct Arr
{
    py::object keep; // owner of the memory
    bool device = false;
    void *ptr = nullptr;
    std::vector<size_t> shape;
    Kind kind = Kind::C128;
    size_t ndim() const
    {
        return shape.size();
    }
    size_t size() const
    {
        size_t s = 1;
        for (size_t e : shape)
            s *= e;
        return s;
    }
};

std::string join_sizes(const std::vector<size_t> &v)
{
    std::ostringstream o;
    for (size_t i = 0; i < v.size(); ++i)
        o << (i ? ", " : "") << v[i];
    return o.str();
}

bool is_cuda(py::handle obj)
{
    return py::hasattr(obj, "__cuda_array_interface__");
}

Arr from_cuda(py::handle obj, bool real)
{
    py::dict cai = obj.attr("__cuda_array_interface__");
    Arr a;
    a.keep = py::reinterpret_borrow<py::object>(obj);
    a.device = true;
    for (auto e : cai["shape"].cast<py::tuple>())
        a.shape.push_back(e.cast<size_t>());
    const std::string ts = cai["typestr"].cast<std::string>();
    if (ts == "<c16")
        a.kind = Kind::C128;
    else if (ts == "<c8")
        a.kind = Kind::C64;
    else if (ts == "<f8")
        a.kind = Kind::F64;
    else if (ts == "<f4")
        a.kind = Kind::F32;
    else
        throw py::value_error("unsupported device array dtype " + ts);
    if (real != (a.kind == Kind::F64 || a.kind == Kind::F32))
        throw py::value_error(real ? "expected a real device array" : "expected a complex device array");
    if (!cai.contains("strides") || cai["strides"].is_none())
    {
    }
    else
    {
        const size_t isz = a.kind == Kind::C128 ? 16 : a.kind == Kind::F32 ? 4 : 8;
        std::vector<size_t> got, want(a.shape.size());
        for (auto e : cai["strides"].cast<py::tuple>())
            got.push_back(e.cast<size_t>());
        size_t acc = isz;
        for (size_t i = a.shape.size(); i-- > 0;)
        {
            want[i] = acc;
            acc *= a.shape[i];
        }
        if (got != want)
            throw py::value_error("array MUST have C-style strides");
    }
    a.ptr = reinterpret_cast<void *>(cai["data"].cast<py::tuple>()[0].cast<uintptr_t>());
    return a;
}

// numpy path: complex128 (or float64 for data) C-contiguous host array
Arr from_host(py::handle obj, bool real)
{
    py::module_ np = py::module_::import("numpy");
    py::object want = real ? np.attr("float64") : np.attr("complex128");
    py::array arr;
    if (py::isinstance<py::array>(obj) && py::reinterpret_borrow<py::array>(obj).dtype().is(py::dtype::from_args(want)))
    {
        arr = py::reinterpret_borrow<py::array>(obj);
        if (!(arr.flags() & py::array::c_style))
        {
            std::vector<size_t> shape, strides, expect(arr.ndim());
            for (py::ssize_t i = 0; i < arr.ndim(); ++i)
            {
                shape.push_back((size_t)arr.shape(i));
                strides.push_back((size_t)arr.strides(i) / arr.itemsize());
            }
            size_t acc = 1;
            for (size_t i = shape.size(); i-- > 0;)
            {
                expect[i] = acc;
                acc *= shape[i];
            }
            throw py::value_error("ndarray MUST have C-style strides.\nExpected strides: " + join_sizes(expect) +
                                  "\nGot strides:      " + join_sizes(strides) + "\nShape:            " +
                                  join_sizes(shape));
        }
    }
    else
    {
        arr = np.attr("ascontiguousarray")(np.attr("asarray")(obj, "dtype"_a = want));
    }
    Arr a;
    a.keep = arr;
    a.ptr = arr.mutable_data();
    for (py::ssize_t i = 0; i < arr.ndim(); ++i)
        a.shape.push_back((size_t)arr.shape(i));
    a.kind = real ? Kind::F64 : Kind::C128;
    return a;
}

Arr get_states(py::handle obj)
{
    return is_cuda(obj) ? from_cuda(obj, false) : from_host(obj, false);
}

Arr get_data(py::handle obj, const Arr &like)
{
    if (like.device)
    {
        if (!is_cuda(obj))
            throw py::value_error("data must be on the same device as the states");
        Arr d = from_cuda(obj, true);
        if ((like.kind == Kind::C128) != (d.kind == Kind::F64))
            throw py::value_error("data must be float64 for complex128 states and float32 for complex64 states");
        return d;
    }
    return from_host(obj, true);
}

// new zero array shaped `shape`, same family (numpy / device tensor) and precision as `like`
Arr new_zeros(const Arr &like, const std::vector<size_t> &shape)
{
    Arr o;
    o.shape = shape;
    o.kind = like.kind;
    o.device = like.device;
    if (like.device)
    {
        py::tuple t(shape.size());
        for (size_t i = 0; i < shape.size(); ++i)
            t[i] = py::int_(shape[i]);
        if (!py::hasattr(like.keep, "new_zeros"))
            throw py::value_error("device arrays must be torch tensors (new_zeros is used for results)");
        o.keep = like.keep.attr("new_zeros")(t);
        Arr chk = from_cuda(o.keep, false);
        o.ptr = chk.ptr;
    }
    else
    {
        // numpy.zeros: calloc'd, so a large result is zero pages until the
        // device-to-host copy writes it (no separate zeroing pass)
        py::module_ np = py::module_::import("numpy");
        py::tuple t(shape.size());
        for (size_t i = 0; i < shape.size(); ++i)
            t[i] = py::int_(shape[i]);
        py::array arr = np.attr("zeros")(t, "dtype"_a = np.attr("complex128"));
        o.keep = arr;
        o.ptr = arr.mutable_data();
    }
    return o;
}

// Stream for device arrays: torch's current stream, so results are ordered
// with the caller's torch work.
cudaStream_t torch_stream_for(const Arr &a)
{
    if (!a.device)
        return cudaStreamPerThread;
    py::module_ torch = py::module_::import("torch");
    py::object s = torch.attr("cuda").attr("current_stream")();
    return reinterpret_cast<cudaStream_t>(s.attr("cuda_stream").cast<uintptr_t>());
}

template <typename F> void gpu_call(const Arr &ref, F &&f)
{
    const cudaStream_t st = torch_stream_for(ref);
    py::gil_scoped_release nogil;
    fp::detail::StreamScope scope(st);
    f();
}

// Dispatch on precision: complex128 -> float64 path, complex64 -> mixed path.
#define FPG_DISPATCH(arr, C, ...)                                                                                      \
    do                                                                                                                 \
    {                                                                                                                  \
        if ((arr).kind == Kind::C128)                                                                                  \
        {                                                                                                              \
            using C = cd;                                                                                              \
            __VA_ARGS__;                                                                                               \
        }                                                                                                              \
        else                                                                                                           \
        {                                                                                                              \
            using C = cf;                                                                                              \
            __VA_ARGS__;                                                                                               \
        }                                                                                                              \
    } while (0)

template <typename V> py::array_t<cd> to_numpy_2d(const std::vector<size_t> &shape, V &&fill)
{
    py::array_t<cd> arr(std::vector<py::ssize_t>(shape.begin(), shape.end()));
    std::memset(arr.mutable_data(), 0, arr.nbytes());
    fill(arr.mutable_data());
    return arr;
}

std::vector<cd> coeff_vector(py::handle obj)
{
    Arr a = from_host(obj, false);
    if (a.ndim() != 1)
        throw py::value_error("ndarray_to_mdspan: expected 1 dimensions, got " + std::to_string(a.ndim()));
    const cd *p = (const cd *)a.ptr;
    return std::vector<cd>(p, p + a.size());
}

std::string pstr(const fp::PauliString &s)
{
    return s.str();
}

std::string pauli_str(const fp::Pauli &p)
{
    return std::string(1, p.symbol());
}

using PauliOpD = fp::PauliOp<double>;
using SummedD = fp::SummedPauliOp<double>;

} // namespace

PYBIND11_MODULE(_fast_pauli, m)
{
    m.doc() = "GB300 (sm_103a) implementation of fast_pauli's Pauli string / operator API";

    py::register_exception_translator([](std::exception_ptr p) {
        try
        {
            if (p)
                std::rethrow_exception(p);
        }
        catch (const std::invalid_argument &e)
        {
            PyErr_SetString(PyExc_ValueError, e.what());
        }
    });

    // ------------------------------------------------------------------ Pauli
    py::class_<fp::Pauli>(m, "Pauli",
                          "A class for efficient representation of a 2x2 Pauli Matrix sigma_i in {I, X, Y, Z}")
        .def(py::init<>(), "Default constructor to initialize with identity matrix.")
        .def(py::init([](int code) { return fp::Pauli(code); }), "code"_a)
        .def(py::init([](char symbol) { return fp::Pauli(symbol); }), "symbol"_a)
        .def(
            "__matmul__", [](const fp::Pauli &a, const fp::Pauli &b) { return a * b; }, py::is_operator())
        .def("to_tensor",
             [](const fp::Pauli &self) {
                 return to_numpy_2d({2, 2}, [&](cd *p) { self.to_tensor(fp::Span<cd, 2>(p, 2, 2)); });
             })
        .def("clone", [](const fp::Pauli &self) { return fp::Pauli(self); })
        .def("__str__", &pauli_str)
        .def("__repr__", &pauli_str)
        .def(py::pickle([](const fp::Pauli &self) { return (int)self.code; },
                        [](int code) { return fp::Pauli(code); }));

    // ------------------------------------------------------------ PauliString
    py::class_<fp::PauliString>(m, "PauliString")
        .def(py::init<>())
        .def(py::init<const std::string &>(), "string"_a)
        .def(py::init<std::vector<fp::Pauli>>(), "paulis"_a)
        .def("__str__", &pstr)
        .def("__repr__", &pstr)
        .def(
            "__matmul__", [](const fp::PauliString &a, const fp::PauliString &b) { return a * b; },
            py::is_operator())
        .def(
            "__add__",
            [](const fp::PauliString &a, const fp::PauliString &b) { return PauliOpD(std::vector<fp::PauliString>{a, b}); },
            py::is_operator())
        .def(
            "__sub__",
            [](const fp::PauliString &a, const fp::PauliString &b) {
                return PauliOpD(std::vector<cd>{1.0, -1.0}, std::vector<fp::PauliString>{a, b});
            },
            py::is_operator())
        .def_property_readonly("n_qubits", &fp::PauliString::n_qubits)
        .def_property_readonly("dim", &fp::PauliString::dim)
        .def_property_readonly("weight", [](const fp::PauliString &s) { return (int)s.weight; })
        .def(
            "apply",
            [](const fp::PauliString &self, py::object states, cd coeff) -> py::object {
                Arr in = get_states(states);
                if (in.ndim() == 1)
                {
                    if (in.size() != self.dim())
                        throw py::value_error("Input vector size must match the number of qubits");
                    Arr out = new_zeros(in, in.shape);
                    // the reference's 1-D path ignores coeff (__pauli_string_bindings.hpp:142)
                    FPG_DISPATCH(in, C, gpu_call(in, [&] {
                                     self.run_apply<C>((C *)out.ptr, (const C *)in.ptr, 1, C(1), true);
                                 }));
                    return out.keep;
                }
                if (in.ndim() == 2)
                {
                    if (in.shape[0] != self.dim())
                        throw py::value_error("[PauliString] states shape (" + std::to_string(in.shape[0]) +
                                              ") must match the dimension of the operators (" +
                                              std::to_string(self.dim()) + ")");
                    Arr out = new_zeros(in, in.shape);
                    FPG_DISPATCH(in, C, gpu_call(in, [&] {
                                     self.run_apply<C>((C *)out.ptr, (const C *)in.ptr, in.shape[1], C(coeff), true);
                                 }));
                    return out.keep;
                }
                throw py::value_error("apply: expected 1 or 2 dimensions, got " + std::to_string(in.ndim()));
            },
            "states"_a, "coeff"_a = cd(1.0))
        .def(
            "expectation_value",
            [](const fp::PauliString &self, py::object states, cd coeff) -> py::object {
                Arr in = get_states(states);
                if (in.ndim() != 1 && in.ndim() != 2)
                    throw py::value_error("expectation_value: expected 1 or 2 dimensions, got " +
                                          std::to_string(in.ndim()));
                const size_t S = in.ndim() == 1 ? 1 : in.shape[1];
                if (in.shape[0] != self.dim())
                    throw py::value_error("[PauliString] states shape (" + std::to_string(in.shape[0]) +
                                          ") must match the dimension of the operators (" + std::to_string(self.dim()) +
                                          ")");
                Arr out = new_zeros(in, {S});
                FPG_DISPATCH(in, C, gpu_call(in, [&] {
                                 self.run_expect<C>((C *)out.ptr, (const C *)in.ptr, S, C(coeff), true);
                             }));
                return out.keep;
            },
            "states"_a, "coeff"_a = cd(1.0))
        .def("to_tensor",
             [](const fp::PauliString &self) {
                 const size_t D = self.dim();
                 return to_numpy_2d({D, D}, [&](cd *p) {
                     if (D)
                         self.to_tensor(fp::Span<cd, 2>(p, D, D));
                 });
             })
        .def("clone", [](const fp::PauliString &self) { return fp::PauliString(self); })
        .def(py::pickle([](const fp::PauliString &self) { return self.paulis; },
                        [](std::vector<fp::Pauli> paulis) { return fp::PauliString(std::move(paulis)); }));

    // ----------------------------------------------------------------- PauliOp
    py::class_<PauliOpD>(m, "PauliOp")
        .def(py::init<>())
        .def(py::init<const std::vector<std::string> &>(), "pauli_strings"_a)
        .def(py::init<std::vector<fp::PauliString>>(), "pauli_strings"_a)
        .def(py::init([](py::array coefficients, std::vector<fp::PauliString> pauli_strings) {
                 return PauliOpD(coeff_vector(coefficients), std::move(pauli_strings));
             }),
             "coefficients"_a, "pauli_strings"_a)
        .def(py::init([](std::vector<cd> coefficients, std::vector<fp::PauliString> pauli_strings) {
                 return PauliOpD(std::move(coefficients), std::move(pauli_strings));
             }),
             "coefficients"_a, "pauli_strings"_a)
        .def(py::init([](std::vector<cd> coefficients, const std::vector<std::string> &strings) {
                 std::vector<fp::PauliString> ps;
                 for (auto const &s : strings)
                     ps.emplace_back(s);
                 return PauliOpD(std::move(coefficients), std::move(ps));
             }),
             "coefficients"_a, "pauli_strings"_a)
        .def(py::init([](py::array coefficients, const std::vector<std::string> &strings) {
                 std::vector<fp::PauliString> ps;
                 for (auto const &s : strings)
                     ps.emplace_back(s);
                 return PauliOpD(coeff_vector(coefficients), std::move(ps));
             }),
             "coefficients"_a, "pauli_strings"_a)
        .def(
            "__matmul__", [](const PauliOpD &a, const PauliOpD &b) { return a * b; }, py::is_operator())
        .def(
            "__matmul__", [](const PauliOpD &a, const fp::PauliString &b) { return a * b; }, py::is_operator())
        .def(
            "__rmatmul__", [](const PauliOpD &self, const fp::PauliString &lhs) { return lhs * self; },
            py::is_operator())
        .def(
            "__mul__",
            [](const PauliOpD &self, cd rhs) {
                PauliOpD r(self);
                r.scale(rhs);
                return r;
            },
            py::is_operator())
        .def(
            "__rmul__",
            [](const PauliOpD &self, cd lhs) {
                PauliOpD r(self);
                r.scale(lhs);
                return r;
            },
            py::is_operator())
        .def(
            "__imul__",
            [](PauliOpD &self, cd f) -> PauliOpD & {
                self.scale(f);
                return self;
            },
            py::is_operator())
        .def(
            "__add__",
            [](const PauliOpD &a, const PauliOpD &b) {
                PauliOpD r(a);
                r.extend(b);
                return r;
            },
            py::is_operator())
        .def(
            "__add__",
            [](const PauliOpD &a, const fp::PauliString &b) {
                PauliOpD r(a);
                r.extend(b, 1);
                return r;
            },
            py::is_operator())
        .def(
            "__radd__",
            [](const PauliOpD &self, const fp::PauliString &lhs) {
                PauliOpD r(self);
                r.extend(lhs, 1);
                return r;
            },
            py::is_operator())
        .def(
            "__iadd__",
            [](PauliOpD &self, const PauliOpD &o) -> PauliOpD & {
                self.extend(o);
                return self;
            },
            py::is_operator())
        .def(
            "__iadd__",
            [](PauliOpD &self, const fp::PauliString &o) -> PauliOpD & {
                self.extend(o, 1);
                return self;
            },
            py::is_operator())
        .def(
            "__sub__",
            [](const PauliOpD &a, const PauliOpD &b) {
                PauliOpD r(a);
                r.extend(-b);
                return r;
            },
            py::is_operator())
        .def(
            "__sub__",
            [](const PauliOpD &a, const fp::PauliString &b) {
                PauliOpD r(a);
                r.extend(b, -1);
                return r;
            },
            py::is_operator())
        .def(
            "__rsub__",
            [](const PauliOpD &self, const fp::PauliString &lhs) {
                PauliOpD r(-self);
                r.extend(lhs, 1);
                return r;
            },
            py::is_operator())
        .def(
            "__isub__",
            [](PauliOpD &self, const PauliOpD &o) -> PauliOpD & {
                self.extend(-o);
                return self;
            },
            py::is_operator())
        .def(
            "__isub__",
            [](PauliOpD &self, const fp::PauliString &o) -> PauliOpD & {
                self.extend(o, -1);
                return self;
            },
            py::is_operator())
        .def(
            "extend", [](PauliOpD &self, const PauliOpD &other) { self.extend(other); }, "other"_a)
        .def(
            "extend",
            [](PauliOpD &self, const fp::PauliString &other, cd multiplier, bool dedupe) {
                self.extend(other, multiplier, dedupe);
            },
            "other"_a, "multiplier"_a, "dedupe"_a = true)
        .def_property_readonly("dim", &PauliOpD::dim)
        .def_property_readonly("n_qubits", &PauliOpD::n_qubits)
        .def_property_readonly("n_pauli_strings", &PauliOpD::n_pauli_strings)
        .def_property_readonly("coeffs", [](const PauliOpD &self) { return self.coeffs; })
        .def_property_readonly("pauli_strings", [](const PauliOpD &self) { return self.pauli_strings; })
        .def_property_readonly("pauli_strings_as_str",
                               [](const PauliOpD &self) {
                                   std::vector<std::string> v;
                                   for (auto const &p : self.pauli_strings)
                                       v.push_back(p.str());
                                   return v;
                               })
        .def(
            "scale", [](PauliOpD &self, cd factor) { self.scale(factor); }, "factor"_a)
        .def(
            "scale",
            [](PauliOpD &self, py::array factors) {
                std::vector<cd> f = coeff_vector(factors);
                self.scale(fp::Span<cd, 1>(f.data(), f.size()));
            },
            "factors"_a)
        .def(
            "apply",
            [](const PauliOpD &self, py::object states) -> py::object {
                Arr in = get_states(states);
                if (in.ndim() != 1 && in.ndim() != 2)
                    throw py::value_error("apply: expected 1 or 2 dimensions, got " + std::to_string(in.ndim()));
                const size_t S = in.ndim() == 1 ? 1 : in.shape[1];
                if (in.shape[0] != self.dim())
                    throw py::value_error("[PauliOp] state size must match the dimension of the operators");
                Arr out = new_zeros(in, in.shape);
                FPG_DISPATCH(in, C, gpu_call(in, [&] {
                                 self.run_apply<C>((C *)out.ptr, (const C *)in.ptr, S, true);
                             }));
                return out.keep;
            },
            "states"_a)
        .def(
            "expectation_value",
            [](const PauliOpD &self, py::object states) -> py::object {
                Arr in = get_states(states);
                if (in.ndim() != 1 && in.ndim() != 2)
                    throw py::value_error("expectation_value: expected 1 or 2 dimensions, got " +
                                          std::to_string(in.ndim()));
                const size_t S = in.ndim() == 1 ? 1 : in.shape[1];
                if (in.shape[0] != self.dim())
                    throw py::value_error("[PauliOp] state size must match the dimension of the operators");
                Arr out = new_zeros(in, {S});
                FPG_DISPATCH(in, C, gpu_call(in, [&] {
                                 self.run_expect<C>((C *)out.ptr, (const C *)in.ptr, S, true);
                             }));
                return out.keep;
            },
            "states"_a)
        .def("to_tensor",
             [](const PauliOpD &self) {
                 const size_t D = self.dim();
                 return to_numpy_2d({D, D}, [&](cd *p) {
                     if (D)
                         self.to_tensor(fp::Span<cd, 2>(p, D, D));
                 });
             })
        .def("clone", [](const PauliOpD &self) { return PauliOpD(self); })
        .def(py::pickle([](const PauliOpD &self) { return py::make_tuple(self.coeffs, self.pauli_strings); },
                        [](py::tuple t) {
                            return PauliOpD(t[0].cast<std::vector<cd>>(), t[1].cast<std::vector<fp::PauliString>>());
                        }));

    // ----------------------------------------------------------- SummedPauliOp
    auto summed_from = [](std::vector<fp::PauliString> ps, py::handle coeffs) {
        Arr c = from_host(coeffs, false);
        if (c.ndim() != 2)
            throw py::value_error("ndarray_to_mdspan: expected 2 dimensions, got " + std::to_string(c.ndim()));
        return SummedD(ps, fp::Span<cd, 2>((cd *)c.ptr, c.shape[0], c.shape[1]));
    };
    py::class_<SummedD>(m, "SummedPauliOp")
        .def(py::init<>())
        .def(py::init([summed_from](std::vector<fp::PauliString> pauli_strings, py::array coeffs) {
                 return summed_from(std::move(pauli_strings), coeffs);
             }),
             "pauli_strings"_a, "coeffs"_a)
        .def(py::init([summed_from](const std::vector<std::string> &pauli_strings, py::array coeffs) {
                 std::vector<fp::PauliString> ps;
                 for (auto const &s : pauli_strings)
                     ps.emplace_back(s);
                 return summed_from(std::move(ps), coeffs);
             }),
             "pauli_strings"_a, "coeffs"_a)
        .def_property_readonly("dim", &SummedD::dim)
        .def_property_readonly("n_operators", &SummedD::n_operators)
        .def_property_readonly("n_pauli_strings", &SummedD::n_pauli_strings)
        .def_property(
            "coeffs",
            [](const SummedD &self) {
                const size_t P = self.coeffs.extent(0), K = self.coeffs.extent(1);
                return to_numpy_2d({K, P}, [&](cd *p) {
                    for (size_t i = 0; i < P; ++i)
                        for (size_t j = 0; j < K; ++j)
                            p[j * P + i] = self.coeffs(i, j);
                });
            },
            [](SummedD &self, py::object coeffs_new) {
                Arr c = from_host(coeffs_new, false);
                if (c.ndim() != 2 || c.shape[0] != self.n_operators() || c.shape[1] != self.n_pauli_strings())
                    throw py::value_error(
                        "The shape of provided coeffs must match the number of operators and PauliStrings");
                const cd *p = (const cd *)c.ptr;
                const size_t P = self.coeffs.extent(0), K = self.coeffs.extent(1);
                for (size_t i = 0; i < P; ++i)
                    for (size_t j = 0; j < K; ++j)
                        self.coeffs(i, j) = p[j * P + i];
            })
        .def_property_readonly("pauli_strings", [](const SummedD &self) { return self.pauli_strings; })
        .def_property_readonly("pauli_strings_as_str",
                               [](const SummedD &self) {
                                   std::vector<std::string> v;
                                   for (auto const &p : self.pauli_strings)
                                       v.push_back(p.str());
                                   return v;
                               })
        .def(
            "apply",
            [](const SummedD &self, py::object states) -> py::object {
                Arr in = get_states(states);
                if (in.ndim() != 1 && in.ndim() != 2)
                    throw py::value_error("apply: expected 1 or 2 dimensions, got " + std::to_string(in.ndim()));
                const size_t S = in.ndim() == 1 ? 1 : in.shape[1];
                if (in.shape[0] != self.dim())
                    throw py::value_error("state size must match the dimension of the operators");
                Arr out = new_zeros(in, in.shape);
                FPG_DISPATCH(in, C, gpu_call(in, [&] {
                                 self.run_apply<C>((C *)out.ptr, (const C *)in.ptr, S, true);
                             }));
                return out.keep;
            },
            "states"_a)
        .def(
            "apply_weighted",
            [](const SummedD &self, py::object states, py::object data) -> py::object {
                Arr in = get_states(states);
                if (in.ndim() != 1 && in.ndim() != 2)
                    throw py::value_error("apply_weighted: expected 1 or 2 dimensions for states, got " +
                                          std::to_string(in.ndim()));
                Arr d = get_data(data, in);
                const size_t S = in.ndim() == 1 ? 1 : in.shape[1];
                const size_t dK = d.ndim() >= 1 ? d.shape[0] : 0;
                const size_t dS = d.ndim() == 2 ? d.shape[1] : 1;
                if (d.ndim() != in.ndim())
                    throw py::value_error("ndarray_to_mdspan: expected " + std::to_string(in.ndim()) +
                                          " dimensions, got " + std::to_string(d.ndim()));
                if (dK != self.n_operators() || dS != S)
                    throw py::value_error("data(k,t) must have the same number of operators as the SummedPauliOp "
                                          "and the same number of states as the input states");
                if (in.shape[0] != self.dim())
                    throw py::value_error("state size must match the dimension of the operators");
                Arr out = new_zeros(in, in.shape);
                FPG_DISPATCH(in, C, gpu_call(in, [&] {
                                 using R = typename C::value_type;
                                 self.run_apply_weighted<C, R>((C *)out.ptr, (const C *)in.ptr, (const R *)d.ptr, S,
                                                               true);
                             }));
                return out.keep;
            },
            "states"_a, "data"_a)
        .def(
            "expectation_value",
            [](const SummedD &self, py::object states) -> py::object {
                Arr in = get_states(states);
                if (in.ndim() != 1 && in.ndim() != 2)
                    throw py::value_error("expectation_value: expected 1 or 2 dimensions for states, got " +
                                          std::to_string(in.ndim()));
                const size_t S = in.ndim() == 1 ? 1 : in.shape[1];
                if (in.shape[0] != self.dim())
                    throw py::value_error("states must have the same dimension (" + std::to_string(in.shape[0]) +
                                          ") as the SummedPauliOp (" + std::to_string(self.dim()) + ")");
                std::vector<size_t> oshape = in.ndim() == 1 ? std::vector<size_t>{self.n_operators()}
                                                             : std::vector<size_t>{self.n_operators(), S};
                Arr out = new_zeros(in, oshape);
                FPG_DISPATCH(in, C, gpu_call(in, [&] {
                                 self.run_expect<C>((C *)out.ptr, (const C *)in.ptr, S, true);
                             }));
                return out.keep;
            },
            "states"_a)
        .def("to_tensor",
             [](const SummedD &self) {
                 const size_t D = self.dim(), K = self.n_operators();
                 py::array_t<cd> arr({(py::ssize_t)K, (py::ssize_t)D, (py::ssize_t)D});
                 std::memset(arr.mutable_data(), 0, arr.nbytes());
                 if (D && K)
                     self.to_tensor(fp::Span<cd, 3>(arr.mutable_data(), K, D, D));
                 return arr;
             })
        .def("clone", [](const SummedD &self) { return SummedD(self.pauli_strings, self.coeffs_raw); })
        .def("split", &SummedD::split)
        .def("square", &SummedD::square)
        .def(py::pickle([](const SummedD &self) { return py::make_tuple(self.pauli_strings, self.coeffs_raw); },
                        [](py::tuple t) {
                            return SummedD(t[0].cast<std::vector<fp::PauliString>>(), t[1].cast<std::vector<cd>>());
                        }));

    m.def("release_cached_memory", &fp::release_cached_memory,
          "Return the device memory the library keeps for reuse by later calls to the device.");

    // ----------------------------------------------------------------- helpers
    auto helpers = m.def_submodule("helpers");
    helpers.def("get_nontrivial_paulis", &fp::get_nontrivial_paulis, "weight"_a);
    helpers.def("calculate_pauli_strings", &fp::calculate_pauli_strings, "n_qubits"_a, "weight"_a);
    helpers.def("calculate_pauli_strings_max_weight", &fp::calculate_pauli_strings_max_weight, "n_qubits"_a,
                "weight"_a);
    helpers.def(
        "pauli_string_sparse_repr",
        [](const std::vector<fp::Pauli> &paulis) {
            py::gil_scoped_release nogil;
            return fp::get_sparse_repr<double>(paulis);
        },
        "paulis"_a);
}
