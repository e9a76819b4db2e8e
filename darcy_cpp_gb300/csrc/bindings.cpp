// Python extension `_core`: the reference's pybind11 surface (darcy-cpp
// src/bindings.cpp:96-271, stub python/darcy/_core.pyi) over the C ABI of
// libdarcy_gpu.so. Same functions, keyword names, defaults, result type and
// InvalidInput(ValueError) messages; the compute runs on the GPU with the GIL
// released. Additive keywords: form ("fp64" | "mixed") and x0 (warm start),
// plus solve_batch_uneven and gpu_info.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/darcy_gpu.h"

namespace py = pybind11;

namespace {

using Array = py::array_t<double, py::array::c_style | py::array::forcecast>;

struct InvalidInput : std::invalid_argument {
    using std::invalid_argument::invalid_argument;
};

dgpu_context* context() {
    static std::once_flag once;
    static dgpu_context* ctx = nullptr;
    static int rc = 0;
    static std::string err;
    std::call_once(once, [] {
        rc = dgpu_create(-1, &ctx);
        if (rc != DGPU_OK) err = dgpu_last_error();
    });
    if (!ctx) throw std::runtime_error("darcy GPU engine unavailable: " + err);
    return ctx;
}

void check(int rc) {
    if (rc == DGPU_OK) return;
    const std::string msg = dgpu_last_error();
    if (rc == DGPU_INVALID_INPUT) throw InvalidInput(msg);
    throw std::runtime_error(msg);
}

int preconditioner_code(const std::string& name) {  // solver.hpp:182-187
    if (name == "multigrid" || name == "mg") return DGPU_PC_MULTIGRID;
    if (name == "jacobi") return DGPU_PC_JACOBI;
    if (name == "none") return DGPU_PC_NONE;
    throw InvalidInput("unknown preconditioner '" + name + "'; expected one of: multigrid, jacobi, none");
}

int form_code(const std::string& name) {
    if (name == "fp64" || name == "plain") return DGPU_FORM_FP64;
    if (name == "mixed") return DGPU_FORM_MIXED;
    throw InvalidInput("unknown form '" + name + "'; expected one of: fp64, mixed");
}

// bindings.cpp:33-48
dgpu_options make_options(double tol, int max_iter, const std::string& pc, int pre, int post, int cycle,
                          bool history, const std::string& form) {
    dgpu_options o{};
    o.tol = tol;
    o.max_iter = max_iter;
    o.preconditioner = preconditioner_code(pc);
    o.pre_sweeps = pre;
    o.post_sweeps = post;
    o.cycle_index = cycle;
    o.record_history = history ? 1 : 0;
    o.form = form_code(form);
    if (!(tol > 0.0)) throw InvalidInput("tol must be positive");            // solver.hpp:86
    if (max_iter < 1) throw InvalidInput("max_iter must be at least 1");     // solver.hpp:87
    if (pre < 1 || post < 1) throw InvalidInput("pre_sweeps and post_sweeps must be at least 1");
    if (cycle < 1 || cycle > 2) throw InvalidInput("cycle_index must be 1 (V-cycle) or 2 (W-cycle)");
    return o;
}

int64_t require_square_2d(const py::buffer_info& buf, const char* what) {  // bindings.cpp:73-78
    if (buf.ndim != 2 || buf.shape[0] != buf.shape[1] || buf.shape[0] < 1)
        throw InvalidInput(std::string(what) + " must be a square 2-D array with at least one cell");
    return (int64_t)buf.shape[0];
}

bool is_array_like(const py::object& f) {
    return py::isinstance<py::array>(f) || py::isinstance<py::list>(f) || py::isinstance<py::tuple>(f);
}

// bindings.cpp:51-63: f is a scalar or an (n, n) array. Returns an empty
// vector for a scalar (passed separately).
std::vector<double> make_rhs(const py::object& f, int64_t n, double& scalar) {
    if (is_array_like(f)) {
        Array arr = py::cast<Array>(f);
        auto buf = arr.request();
        if (buf.ndim != 2 || buf.shape[0] != n || buf.shape[1] != n)
            throw InvalidInput("f must be a scalar or an array with the same shape as a");
        const double* p = static_cast<const double*>(buf.ptr);
        scalar = 0.0;
        return std::vector<double>(p, p + n * n);
    }
    scalar = py::cast<double>(f);
    return {};
}

std::vector<double> make_x0(const py::object& x0, const std::vector<int64_t>& shape) {
    if (x0.is_none()) return {};
    Array arr = py::cast<Array>(x0);
    auto buf = arr.request();
    bool ok = buf.ndim == (py::ssize_t)shape.size();
    for (size_t q = 0; ok && q < shape.size(); ++q) ok = buf.shape[q] == shape[q];
    if (!ok) throw InvalidInput("x0 must have the same shape as a");
    const double* p = static_cast<const double*>(buf.ptr);
    size_t count = 1;
    for (int64_t s : shape) count *= (size_t)s;
    return std::vector<double>(p, p + count);
}

py::array_t<double> new_array(std::vector<py::ssize_t> shape) { return py::array_t<double>(shape); }

// Per-problem results as numpy arrays (int64 counts, float64 residuals, bool
// flags) filled from the C ABI's buffers: a Python list per field cost
// ~0.1 ms per thousand problems, twice (list, then array).
py::array_t<int64_t> int64_array(const std::vector<int>& v) {
    py::array_t<int64_t> out((py::ssize_t)v.size());
    int64_t* p = out.mutable_data();
    for (size_t k = 0; k < v.size(); ++k) p[k] = v[k];
    return out;
}
py::array_t<bool> bool_array(const std::vector<int>& v) {
    py::array_t<bool> out((py::ssize_t)v.size());
    bool* p = out.mutable_data();
    for (size_t k = 0; k < v.size(); ++k) p[k] = v[k] != 0;
    return out;
}
py::array_t<double> double_array(const std::vector<double>& v) {
    py::array_t<double> out((py::ssize_t)v.size());
    if (!v.empty()) std::memcpy(out.mutable_data(), v.data(), sizeof(double) * v.size());
    return out;
}

struct PyResult {  // bindings.cpp:81-92
    py::array_t<double> u;
    int iterations = 0;
    double residual = 0.0;
    bool converged = false;
    int levels = 1;
    std::vector<double> history;
    double true_residual = 0.0;
    double device_ms = 0.0;
};

}  // namespace

PYBIND11_MODULE(_core, m) {
    m.doc() =
        "GB300 engine for the matrix-free multigrid-preconditioned finite-volume Darcy solver.\n"
        "Low-level extension module; prefer the package API.";

    py::register_exception<InvalidInput>(m, "InvalidInput", PyExc_ValueError);

    py::class_<PyResult>(m, "SolveResult", "Outcome of a single Darcy solve.")
        .def_readonly("u", &PyResult::u, "Solution field, shape (n, n).")
        .def_readonly("iterations", &PyResult::iterations, "CG iterations performed.")
        .def_readonly("residual", &PyResult::residual, "Final relative residual.")
        .def_readonly("converged", &PyResult::converged, "True if the tolerance was reached.")
        .def_readonly("levels", &PyResult::levels, "Number of multigrid levels used.")
        .def_readonly("history", &PyResult::history, "Relative residual per iteration, if recorded.")
        .def_readonly("true_residual", &PyResult::true_residual, "||b - A u|| / ||b|| recomputed on the GPU.")
        .def_readonly("device_ms", &PyResult::device_ms, "Device time of the call (CUDA events).")
        .def("__repr__", [](const PyResult& r) {
            return "SolveResult(iterations=" + std::to_string(r.iterations) +
                   ", residual=" + std::to_string(r.residual) + ", converged=" + (r.converged ? "True" : "False") +
                   ", levels=" + std::to_string(r.levels) + ")";
        });

    m.def(
        "solve",
        [](Array a, py::object f, double tol, int max_iter, const std::string& preconditioner, int pre_sweeps,
           int post_sweeps, int cycle_index, bool record_history, const std::string& form, py::object x0) {
            auto buf = a.request();
            const int64_t n = require_square_2d(buf, "a");
            const dgpu_options o = make_options(tol, max_iter, preconditioner, pre_sweeps, post_sweeps,
                                                cycle_index, record_history, form);
            double fs = 0.0;
            const std::vector<double> rhs = make_rhs(f, n, fs);
            const std::vector<double> u0 = make_x0(x0, {n, n});
            const auto* ap = static_cast<const double*>(buf.ptr);
            PyResult res;
            res.u = new_array({(py::ssize_t)n, (py::ssize_t)n});
            double* up = static_cast<double*>(res.u.request().ptr);
            std::vector<double> hist(record_history && max_iter > 0 ? (size_t)max_iter + 1 : 0);
            dgpu_stats st{};
            int rc;
            {
                py::gil_scoped_release release;
                rc = dgpu_solve(context(), ap, rhs.empty() ? nullptr : rhs.data(), fs, n, &o,
                                u0.empty() ? nullptr : u0.data(), up, hist.empty() ? nullptr : hist.data(), &st);
            }
            check(rc);
            res.iterations = st.iterations;
            res.residual = st.residual;
            res.converged = st.converged != 0;
            res.levels = st.levels;
            if (record_history) res.history.assign(hist.begin(), hist.begin() + st.history_len);
            res.true_residual = st.true_residual;
            res.device_ms = st.device_ms;
            return res;
        },
        // the reference's arguments positional-or-keyword as in its binding
        // (src/bindings.cpp:135-137); the additions keyword-only
        py::arg("a"), py::arg("f") = 1.0, py::arg("tol") = 1e-10, py::arg("max_iter") = 10000,
        py::arg("preconditioner") = "multigrid", py::arg("pre_sweeps") = 1, py::arg("post_sweeps") = 1,
        py::arg("cycle_index") = 2, py::arg("record_history") = false, py::kw_only(), py::arg("form") = "fp64",
        py::arg("x0") = py::none(), "Solve -div(a grad u) = f with homogeneous Dirichlet boundary conditions.");

    m.def(
        "solve_batch",
        [](Array a, py::object f, double tol, int max_iter, const std::string& preconditioner, int pre_sweeps,
           int post_sweeps, int cycle_index, int threads, const std::string& form, py::object x0) {
            (void)threads;  // the GPU engine schedules samples itself
            auto buf = a.request();
            if (buf.ndim != 3 || buf.shape[1] != buf.shape[2] || buf.shape[1] < 1)
                throw InvalidInput("a must have shape (batch, n, n)");
            const int64_t batch = buf.shape[0], n = buf.shape[1];
            const dgpu_options o =
                make_options(tol, max_iter, preconditioner, pre_sweeps, post_sweeps, cycle_index, false, form);
            double fs = 0.0;
            const std::vector<double> rhs = make_rhs(f, n, fs);
            const std::vector<double> u0 = make_x0(x0, {batch, n, n});
            py::array_t<double> out = new_array({(py::ssize_t)batch, (py::ssize_t)n, (py::ssize_t)n});
            std::vector<int> iters((size_t)batch), conv((size_t)batch);
            std::vector<double> res((size_t)batch);
            if (batch > 0) {
                const auto* ap = static_cast<const double*>(buf.ptr);
                double* up = static_cast<double*>(out.request().ptr);
                int rc;
                {
                    py::gil_scoped_release release;
                    rc = dgpu_solve_batch(context(), ap, rhs.empty() ? nullptr : rhs.data(), fs, 0, batch, n, &o,
                                          u0.empty() ? nullptr : u0.data(), up, iters.data(), res.data(),
                                          conv.data(), nullptr);
                }
                check(rc);
            }
            return py::make_tuple(out, int64_array(iters), double_array(res), bool_array(conv));
        },
        // as the reference's binding (src/bindings.cpp:194-196); the additions keyword-only
        py::arg("a"), py::arg("f") = 1.0, py::arg("tol") = 1e-10, py::arg("max_iter") = 10000,
        py::arg("preconditioner") = "multigrid", py::arg("pre_sweeps") = 1, py::arg("post_sweeps") = 1,
        py::arg("cycle_index") = 2, py::arg("threads") = 0, py::kw_only(), py::arg("form") = "fp64",
        py::arg("x0") = py::none(), "Solve a batch of independent Darcy problems, one GPU launch for the whole batch.");

    m.def(
        "solve_batch_uneven",
        [](py::list fields, py::object f, double tol, int max_iter, const std::string& preconditioner,
           int pre_sweeps, int post_sweeps, int cycle_index, const std::string& form, py::object x0) {
            const int64_t count = (int64_t)py::len(fields);
            if (count < 1) throw InvalidInput("need at least one field");
            const dgpu_options o =
                make_options(tol, max_iter, preconditioner, pre_sweeps, post_sweeps, cycle_index, false, form);
            std::vector<int64_t> sides((size_t)count);
            std::vector<double> packed, fpacked, u0packed;
            std::vector<Array> keep;
            keep.reserve((size_t)count);
            double fs = 0.0;
            const bool f_list = py::isinstance<py::list>(f) && py::len(f) == (size_t)count && count > 0 &&
                                !py::isinstance<py::float_>(py::list(f)[0]);
            if (!f_list) fs = py::cast<double>(f);
            py::list x0l;
            if (!x0.is_none()) {
                x0l = py::cast<py::list>(x0);
                if ((int64_t)py::len(x0l) != count) throw InvalidInput("x0 must hold one array per field");
            }
            // sizes first, so the packed input is allocated once (no regrowth
            // of a multi-GB buffer)
            size_t total = 0;
            for (int64_t q = 0; q < count; ++q) {
                keep.push_back(py::cast<Array>(fields[q]));
                auto buf = keep.back().request();
                const int64_t n = require_square_2d(buf, "each field");
                sides[q] = n;
                total += (size_t)(n * n);
            }
            packed.reserve(total);
            if (f_list) fpacked.reserve(total);
            if (!x0.is_none()) u0packed.reserve(total);
            for (int64_t q = 0; q < count; ++q) {
                auto buf = keep[(size_t)q].request();
                const int64_t n = sides[q];
                const auto* p = static_cast<const double*>(buf.ptr);
                packed.insert(packed.end(), p, p + n * n);
                if (f_list) {
                    double dummy;
                    const std::vector<double> r = make_rhs(py::list(f)[q], n, dummy);
                    if (r.empty()) fpacked.insert(fpacked.end(), (size_t)(n * n), dummy);
                    else fpacked.insert(fpacked.end(), r.begin(), r.end());
                }
                if (!x0.is_none()) {
                    const std::vector<double> v = make_x0(x0l[q], {n, n});
                    u0packed.insert(u0packed.end(), v.begin(), v.end());
                }
            }
            // the solutions land in one array; each problem's u is a view of it
            py::array_t<double> ubig = new_array({(py::ssize_t)total});
            double* up = static_cast<double*>(ubig.request().ptr);
            std::vector<double> res((size_t)count);
            std::vector<int> iters((size_t)count), conv((size_t)count), levels((size_t)count);
            int rc;
            {
                py::gil_scoped_release release;
                rc = dgpu_solve_uneven(context(), count, sides.data(), packed.data(),
                                       fpacked.empty() ? nullptr : fpacked.data(), fs, &o,
                                       u0packed.empty() ? nullptr : u0packed.data(), up, iters.data(),
                                       res.data(), conv.data(), levels.data());
            }
            check(rc);
            py::list us;
            size_t off = 0;
            for (int64_t q = 0; q < count; ++q) {
                const py::ssize_t n = (py::ssize_t)sides[q];
                us.append(py::array_t<double>({n, n}, {n * (py::ssize_t)sizeof(double), (py::ssize_t)sizeof(double)},
                                              up + off, ubig));
                off += (size_t)(n * n);
            }
            return py::make_tuple(us, int64_array(iters), double_array(res), bool_array(conv), int64_array(levels));
        },
        py::arg("fields"), py::arg("f") = 1.0, py::kw_only(), py::arg("tol") = 1e-10, py::arg("max_iter") = 10000,
        py::arg("preconditioner") = "multigrid", py::arg("pre_sweeps") = 1, py::arg("post_sweeps") = 1,
        py::arg("cycle_index") = 2, py::arg("form") = "fp64", py::arg("x0") = py::none(),
        "Solve independent problems of different grid sizes in one GPU launch.");

    m.def(
        "apply_operator",
        [](Array a, Array x) {
            auto abuf = a.request();
            const int64_t n = require_square_2d(abuf, "a");
            auto xbuf = x.request();
            if (require_square_2d(xbuf, "x") != n) throw InvalidInput("x must have the same shape as a");
            py::array_t<double> y = new_array({(py::ssize_t)n, (py::ssize_t)n});
            double* yp = static_cast<double*>(y.request().ptr);
            int rc;
            {
                py::gil_scoped_release release;
                rc = dgpu_apply_operator(context(), static_cast<const double*>(abuf.ptr),
                                         static_cast<const double*>(xbuf.ptr), n, yp);
            }
            check(rc);
            return y;
        },
        py::arg("a"), py::arg("x"),
        "Apply the finite-volume operator A to x (matrix-free), on the GPU.");

    m.def(
        "apply_preconditioner",
        [](Array a, Array r, int pre_sweeps, int post_sweeps, int cycle_index, const std::string& form) {
            auto abuf = a.request();
            const int64_t n = require_square_2d(abuf, "a");
            auto rbuf = r.request();
            if (require_square_2d(rbuf, "r") != n) throw InvalidInput("r must have the same shape as a");
            const int fc = form_code(form);
            py::array_t<double> z = new_array({(py::ssize_t)n, (py::ssize_t)n});
            double* zp = static_cast<double*>(z.request().ptr);
            int rc;
            {
                py::gil_scoped_release release;
                rc = dgpu_apply_preconditioner(context(), static_cast<const double*>(abuf.ptr),
                                               static_cast<const double*>(rbuf.ptr), n, pre_sweeps, post_sweeps,
                                               cycle_index, fc, zp);
            }
            check(rc);
            return z;
        },
        // as the reference's binding (src/bindings.cpp:242-243); form keyword-only
        py::arg("a"), py::arg("r"), py::arg("pre_sweeps") = 1, py::arg("post_sweeps") = 1,
        py::arg("cycle_index") = 2, py::kw_only(), py::arg("form") = "fp64",
        "Apply one multigrid cycle to r from a zero initial guess, on the GPU.");

    m.def(
        "hierarchy",
        [](Array a) {
            auto buf = a.request();
            const int64_t n = require_square_2d(buf, "a");
            int64_t cap = 0;
            for (int64_t s = n;;) {
                cap += 6 * s * s;
                if (s <= 1) break;
                s = (s + 1) / 2;
            }
            py::array_t<double> out = new_array({(py::ssize_t)cap});
            double* op = static_cast<double*>(out.request().ptr);
            int64_t got;
            {
                py::gil_scoped_release release;
                got = dgpu_hierarchy(context(), static_cast<const double*>(buf.ptr), n, op, cap);
            }
            if (got != cap) check(DGPU_INVALID_INPUT);
            return out;
        },
        py::arg("a"), "Every level's e, w, n, s, diag, inv_diag as built on the GPU (parity hook).");

    m.def("num_threads", [] { return 1; }, "Host threads used by the solver (the GPU engine uses one).");
    m.def("has_openmp", [] { return false; }, "Whether host-side OpenMP is used (it is not).");
    m.def("set_num_threads", [](int) {}, py::arg("threads"), "Accepted for compatibility; no effect.");
    m.def("gpu_info", [] {
        char buf[512];
        check(dgpu_device_info(context(), buf, (int)sizeof buf));
        return std::string(buf);
    });
    m.attr("__version__") = DARCY_VERSION;
    m.attr("__compiler__") = "nvcc " DARCY_NVCC_VERSION " sm_103a + gcc " __VERSION__;
}
