// ffcore_gpu: fastfermion's `propagate`, both overloads, with the propagation
// run by libffg on the GPU.  Compiled against the reference's own headers and
// pybind11, it accepts and returns the reference's own C++ types as registered
// by the reference's `ffcore` module (pybind11 shares registered types between
// modules built with the same pybind11), so
//
//     import fastfermion, ffcore_gpu
//     fastfermion.propagate = ffcore_gpu.propagate
//
// puts the GPU underneath the reference's Python package without touching it.
// The two functions mirror the lambdas bound at src/python_bind.cpp:392-425
// (Pauli: circuit, observable, n_threads=1, maxdegree=None, mincoeff=None,
// topk=0, max_xweight=-1, xtrunc_period=1, batched=True, parallel="auto") and
// src/python_bind.cpp:490-527 (Majorana: circuit, observable, maxdegree=None,
// mincoeff=0): same argument names, defaults and order, same result types,
// errors raised as RuntimeError.  n_threads and parallel select CPU
// strategies in the reference and are accepted and ignored here (every
// strategy gives the same terms), except that an unknown strategy name with
// n_threads > 1 returns the observable unchanged, as
// src/pauli/propagate.h:306-308, 492 does.
#include <pybind11/complex.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <cstdlib>
#include <optional>
#include <stdexcept>
#include <string>
#include <variant>
#include <vector>

#include "ffg.h"
#include "majorana_propagation.h"
#include "pauli/propagate.h"

namespace py = pybind11;
using namespace fastfermion;

namespace {

ffg_ctx* context() {  // one context (one stream) per process
    static ffg_ctx* ctx = [] {
        ffg_ctx* c = nullptr;
        const char* d = std::getenv("FFG_DEVICE");
        if (ffg_create(&c, d ? std::atoi(d) : 0) != FFG_OK) throw std::runtime_error("ffg_create: no usable CUDA device");
        return c;
    }();
    return ctx;
}

void check(int rc) {
    if (rc != FFG_OK) throw std::runtime_error(ffg_last_error(context()));
}

// polynomial -> [4][n] key planes and coefficients
template <typename Poly, typename Words>
void to_planes(const Poly& p, Words words_of, std::vector<uint64_t>& keys, std::vector<double>& re,
               std::vector<double>& im) {
    const size_t n = p.terms.size();
    keys.assign(4 * n, 0);
    re.resize(n);
    im.resize(n);
    size_t i = 0;
    for (const auto& [s, c] : p.terms) {
        const std::array<uint64_t, 4> w = words_of(s);
        for (int k = 0; k < 4; k++) keys[k * n + i] = w[k];
        re[i] = c.real();
        im[i] = c.imag();
        ++i;
    }
}

struct ResultGuard {
    ffg_result* r = nullptr;
    ~ResultGuard() {
        if (r) ffg_result_free(r);
    }
};

PauliPolynomial propagate_pauli(const pauli_gates::Circuit& circuit,
                                const std::variant<PauliString, PauliPolynomial>& observable, int n_threads,
                                const std::optional<int>& maxdegree, const std::optional<ff_float>& mincoeff,
                                int topk, int max_xweight, int xtrunc_period, bool batched,
                                const std::string& parallel) {
    const PauliPolynomial obs =
        observable.index() == 0 ? PauliPolynomial(std::get<0>(observable)) : std::get<1>(observable);
    if (n_threads > 1 && parallel != "auto" && parallel != "serial" && parallel != "omp" && parallel != "sharded")
        return obs;
    std::vector<uint64_t> keys;
    std::vector<double> re, im;
    to_planes(obs, [](const PauliString& s) {
        return std::array<uint64_t, 4>{s.xory.words[0], s.xory.words[1], s.yorz.words[0], s.yorz.words[1]};
    }, keys, re, im);
    std::vector<ffg_pauli_gate> g(circuit.size());
    for (size_t k = 0; k < circuit.size(); ++k) {
        ffg_pauli_gate& t = g[k];
        t = ffg_pauli_gate{};
        if (circuit[k].index() == 1) {
            const auto& r = std::get<pauli_gates::ROT>(circuit[k]);
            t.kind = FFG_ROT;
            t.theta = r.theta;
            t.x[0] = r.ps.xory.words[0];
            t.x[1] = r.ps.xory.words[1];
            t.z[0] = r.ps.yorz.words[0];
            t.z[1] = r.ps.yorz.words[1];
        } else {
            std::visit(
                [&](const auto& c) {
                    using T = std::decay_t<decltype(c)>;
                    if constexpr (std::is_same_v<T, pauli_gates::H>) {
                        t.kind = FFG_H;
                        t.q0 = c.i;
                    } else if constexpr (std::is_same_v<T, pauli_gates::S>) {
                        t.kind = FFG_S;
                        t.q0 = c.i;
                    } else {
                        t.kind = std::is_same_v<T, pauli_gates::CNOT> ? FFG_CNOT
                                 : std::is_same_v<T, pauli_gates::SWAP> ? FFG_SWAP
                                                                         : FFG_CZ;
                        t.q0 = c.i;
                        t.q1 = c.j;
                    }
                },
                std::get<pauli_gates::CliffordGate>(circuit[k]));
        }
    }
    ffg_pauli_params p{};
    p.maxdegree = maxdegree.has_value() ? maxdegree.value() : ff_ulong::DIGITS;
    p.topk = topk;
    p.mincoeff = mincoeff.has_value() ? mincoeff.value() : 0.0;
    p.max_xweight = max_xweight;
    p.xtrunc_period = xtrunc_period;
    p.batched = batched ? 1 : 0;
    p.deterministic = 0;
    ResultGuard r;
    check(ffg_pauli_propagate(context(), keys.data(), re.data(), im.data(), re.size(), g.data(), g.size(), &p, 0,
                              &r.r));
    const size_t m = ffg_result_size(r.r);
    keys.assign(4 * m, 0);
    re.assign(m, 0.0);
    im.assign(m, 0.0);
    if (m) check(ffg_result_copy(r.r, keys.data(), re.data(), im.data()));
    PauliPolynomial out;
    out.terms.reserve(m);
    for (size_t j = 0; j < m; ++j) {
        PauliString s;
        s.xory.words[0] = keys[j];
        s.xory.words[1] = keys[m + j];
        s.yorz.words[0] = keys[2 * m + j];
        s.yorz.words[1] = keys[3 * m + j];
        out.terms[s] = ff_complex(re[j], im[j]);
    }
    return out;
}

MajoranaPolynomial propagate_majorana(const majorana_gates::MajoranaCircuit& circuit,
                                      const std::variant<MajoranaString, MajoranaPolynomial>& observable,
                                      const std::optional<int>& maxdegree, const std::optional<ff_float>& mincoeff) {
    const MajoranaPolynomial obs =
        observable.index() == 0 ? MajoranaPolynomial(std::get<0>(observable)) : std::get<1>(observable);
    std::vector<uint64_t> keys;
    std::vector<double> re, im;
    to_planes(obs, [](const MajoranaString& s) {
        return std::array<uint64_t, 4>{s.alpha.words[0], s.alpha.words[1], s.alpha.words[2], s.alpha.words[3]};
    }, keys, re, im);
    std::vector<ffg_majorana_gate> g(circuit.size());
    for (size_t k = 0; k < circuit.size(); ++k) {
        g[k] = ffg_majorana_gate{};
        for (int w = 0; w < 4; w++) g[k].alpha[w] = circuit[k].ms.alpha.words[w];
        g[k].theta = circuit[k].theta;
        g[k].r = circuit[k]._r ? 1 : 0;
    }
    ffg_majorana_params p{};
    p.has_maxdegree = maxdegree.has_value() ? 1 : 0;
    p.maxdegree = maxdegree.has_value() ? maxdegree.value() : 0;
    p.mincoeff = mincoeff.has_value() ? mincoeff.value() : 0.0;
    p.deterministic = 0;
    ResultGuard r;
    check(ffg_majorana_propagate(context(), keys.data(), re.data(), im.data(), re.size(), g.data(), g.size(), &p, 0,
                                 &r.r));
    const size_t m = ffg_result_size(r.r);
    keys.assign(4 * m, 0);
    re.assign(m, 0.0);
    im.assign(m, 0.0);
    if (m) check(ffg_result_copy(r.r, keys.data(), re.data(), im.data()));
    MajoranaPolynomial out;
    out.terms.clear();
    out.terms.reserve(m);
    for (size_t j = 0; j < m; ++j) {
        MajoranaString s;
        for (int w = 0; w < 4; w++) s.alpha.words[w] = keys[w * m + j];
        out.terms[s] = ff_complex(re[j], im[j]);
    }
    return out;
}

}  // namespace

PYBIND11_MODULE(ffcore_gpu, m) {
    // the reference's module registers the argument and result types
    py::module_::import("fastfermion.ffcore");
    m.doc() = "fastfermion's propagate with the propagation on the GPU (libffg)";
    m.def("propagate", &propagate_pauli, py::arg("circuit"), py::arg("observable"), py::arg("n_threads") = 1,
          py::arg("maxdegree") = py::none(), py::arg("mincoeff") = py::none(), py::arg("topk") = 0,
          py::arg("max_xweight") = -1, py::arg("xtrunc_period") = 1, py::arg("batched") = true,
          py::arg("parallel") = "auto", "Pauli propagation on the GPU (same signature as fastfermion.propagate)");
    m.def("propagate", &propagate_majorana, py::arg("circuit"), py::arg("observable"),
          py::arg("maxdegree") = py::none(), py::arg("mincoeff") = 0,
          "Majorana propagation on the GPU (same signature as fastfermion.propagate)");
}
