// Reference harness: compiles the reference's exafac/cpp_ext headers, unchanged,
// into a Python module `exafac_ref` (built by oracle/build_ref.sh into
// oracle/_ref/).  TEST INFRASTRUCTURE ONLY: it generates golden vectors and pins
// the oracle restatement; nothing in the product imports it.
//
// The class bindings mirror exafac/cpp_ext/py_module.cpp:37-77.  The extra
// methods are determinism hooks the reference lacks:
//   * reseed the samplers' std::mt19937 streams (sampler.hpp:21-22),
//   * replay those streams on copies to export, exactly, the uniforms and the
//     per-mode permutations that KRPDrawSamples consumes
//     (cp_arls_lev.hpp:61-66,141-149; sts_cp.hpp:190-201,239-249),
//   * overwrite the randomly relabelled COO indices (sparse_tensor.hpp:76-95)
//     and inject / read factor matrices and sigma,
//   * call single pieces of the step (dedup, csr_based_spmm, PTSample, pinv)
//     on given inputs.
// Replays require one OpenMP thread (OMP_NUM_THREADS=1): with more threads the
// reference draws from one generator per thread in static chunks.
#include <iostream>
#include <mpi.h>

#include <algorithm>
#include <execution>
#include <cblas.h>
#include <lapacke.h>
#include <omp.h>

#include <pybind11/pybind11.h>
#include <pybind11/numpy.h>
#include <pybind11/stl.h>

#include "common.h"
#include "grid.hpp"
#include "alltoallv_revised.hpp"

#include "distmat.hpp"
#include "low_rank_tensor.hpp"
#include "sparse_tensor.hpp"

#include "als_optimizer.hpp"
#include "exact_als.hpp"
#include "tensor_stationary.hpp"
#include "accumulator_stationary.hpp"

#include "sampler.hpp"
#include "cp_arls_lev.hpp"
#include "exact_leverage_tree.hpp"
#include "sts_cp.hpp"

using namespace std;
namespace py = pybind11;

using f64arr = py::array_t<double, py::array::c_style | py::array::forcecast>;
using u32arr = py::array_t<uint32_t, py::array::c_style | py::array::forcecast>;

static f64arr buffer_rows(Buffer<double>& b, uint64_t rows, uint64_t cols) {
    f64arr out({(py::ssize_t)rows, (py::ssize_t)cols});
    std::copy(b(), b(rows * cols), out.mutable_data());
    return out;
}

static void require_single_stream(Sampler& s) {
    if (s.local_rng.par_gen.size() != 1 || s.global_rng.par_gen.size() != 1) {
        throw std::runtime_error("stream replay needs OMP_NUM_THREADS=1");
    }
}

static void reseed(Sampler& s, uint32_t local_seed, uint32_t global_seed) {
    for (size_t i = 0; i < s.local_rng.par_gen.size(); i++) s.local_rng.par_gen[i].seed(local_seed + (uint32_t)i);
    for (size_t i = 0; i < s.global_rng.par_gen.size(); i++) s.global_rng.par_gen[i].seed(global_seed + (uint32_t)i);
}

// Runs KRPDrawSamples and replays, on copies of the generators, the uniforms it
// consumed.  ARLS-LEV: per sampled mode, J canonical draws from the local
// stream (discrete_distribution::operator() -> generate_canonical<double,53>)
// and one std::shuffle of iota(J) with the global stream.  The one-element
// rank distribution consumes nothing at world size 1.
static py::tuple arls_draw(CP_ARLS_LEV& s, uint64_t J, uint32_t mode) {
    require_single_stream(s);
    std::mt19937 loc = s.local_rng.par_gen[0];
    std::mt19937 glob = s.global_rng.par_gen[0];
    Buffer<uint32_t> samples;
    Buffer<double> weights;
    vector<Buffer<uint32_t>> uniq;
    s.KRPDrawSamples(J, mode, samples, weights, uniq);
    uint64_t N = s.N;
    u32arr out_s({(py::ssize_t)J, (py::ssize_t)N});
    std::copy(samples(), samples(J * N), out_s.mutable_data());
    f64arr out_w({(py::ssize_t)J});
    std::copy(weights(), weights(J), out_w.mutable_data());
    f64arr uni({(py::ssize_t)N, (py::ssize_t)J});
    u32arr perm({(py::ssize_t)N, (py::ssize_t)J});
    std::fill(uni.mutable_data(), uni.mutable_data() + N * J, -1.0);
    std::fill(perm.mutable_data(), perm.mutable_data() + N * J, 0u);
    for (uint64_t i = 0; i < N; i++) {
        if (i == mode) continue;
        // A distribution over fewer than two rows draws nothing
        // (libstdc++ bits/random.tcc:2660-2664, 2703-2704).
        bool draws = s.U[i].true_row_count >= 2;
        for (uint64_t j = 0; draws && j < J; j++) {
            uni.mutable_data()[i * J + j] = std::generate_canonical<double, std::numeric_limits<double>::digits>(loc);
        }
        vector<uint32_t> p(J);
        std::iota(p.begin(), p.end(), 0);
        std::shuffle(p.begin(), p.end(), glob);
        std::copy(p.begin(), p.end(), perm.mutable_data() + i * J);
    }
    return py::make_tuple(out_s, out_w, uni, perm);
}

// STS-CP: per sampled mode k (ascending), J draws for the eigen-tree descent
// then J draws for the row-tree descent, all from the local stream.
static py::tuple sts_draw(STS_CP& s, uint64_t J, uint32_t mode) {
    require_single_stream(s);
    std::mt19937 loc = s.local_rng.par_gen[0];
    Buffer<uint32_t> samples;
    Buffer<double> weights;
    vector<Buffer<uint32_t>> uniq;
    s.KRPDrawSamples(J, mode, samples, weights, uniq);
    uint64_t N = s.N;
    u32arr out_s({(py::ssize_t)J, (py::ssize_t)N});
    std::copy(samples(), samples(J * N), out_s.mutable_data());
    f64arr out_w({(py::ssize_t)J});
    std::copy(weights(), weights(J), out_w.mutable_data());
    f64arr uni({(py::ssize_t)N, (py::ssize_t)2, (py::ssize_t)J});
    std::fill(uni.mutable_data(), uni.mutable_data() + N * 2 * J, -1.0);
    std::uniform_real_distribution<double> dis(0.0, 1.0);
    for (uint64_t k = 0; k < N; k++) {
        if (k == mode) continue;
        for (int t = 0; t < 2; t++)
            for (uint64_t j = 0; j < J; j++) uni.mutable_data()[(k * 2 + t) * J + j] = dis(loc);
    }
    return py::make_tuple(out_s, out_w, uni);
}

// Copies the sampler's generators, so a caller can draw with KRPDrawSamples and
// then let execute_ALS_step redraw exactly the same samples.
struct StreamState {
    std::mt19937 loc, glob;
};
static StreamState save_streams(Sampler& s) {
    require_single_stream(s);
    return StreamState{s.local_rng.par_gen[0], s.global_rng.par_gen[0]};
}
static void restore_streams(Sampler& s, const StreamState& st) {
    s.local_rng.par_gen[0] = st.loc;
    s.global_rng.par_gen[0] = st.glob;
}

PYBIND11_MODULE(exafac_ref, m) {
    py::class_<Grid>(m, "Grid")
        .def(py::init<py::array_t<int>>())
        .def("get_dimension", &Grid::get_dimension);
    py::class_<TensorGrid>(m, "TensorGrid")
        .def(py::init<py::array_t<int>, Grid&>())
        .def_property_readonly("padded_row_counts", [](TensorGrid& t) { return t.padded_row_counts; });
    py::class_<DistMat1D>(m, "DistMat1D").def(py::init<uint64_t, TensorGrid&, uint64_t>());
    py::class_<LowRankTensor>(m, "LowRankTensor")
        .def(py::init<uint64_t, TensorGrid&>())
        .def("test_gram_matrix_computation", &LowRankTensor::test_gram_matrix_computation)
        .def("initialize_factors_deterministic", &LowRankTensor::initialize_factors_deterministic)
        .def("initialize_factors_gaussian_random", &LowRankTensor::initialize_factors_gaussian_random)
        .def("get_factor",
             [](LowRankTensor& t, int i) {
                 DistMat1D& f = t.factors[i];
                 return buffer_rows(f.data, f.true_row_count, f.cols);
             })
        .def("set_factor",
             [](LowRankTensor& t, int i, f64arr a) {
                 DistMat1D& f = t.factors[i];
                 if ((uint64_t)a.shape(0) != f.true_row_count || (uint64_t)a.shape(1) != f.cols)
                     throw std::runtime_error("factor shape mismatch");
                 std::copy(a.data(), a.data() + f.true_row_count * f.cols, f.data());
             })
        .def("get_sigma", [](LowRankTensor& t) { return buffer_rows(t.sigma, 1, t.rank); })
        .def("set_sigma",
             [](LowRankTensor& t, f64arr a) { std::copy(a.data(), a.data() + t.rank, t.sigma()); });
    py::class_<SparseTensor>(m, "SparseTensor")
        .def(py::init<TensorGrid&, py::array_t<uint32_t>, py::array_t<double>, std::string>())
        .def(py::init<TensorGrid&, uint64_t, uint64_t, uint64_t>())
        .def_readonly("tensor_norm", &SparseTensor::tensor_norm)
        .def("set_indices",
             [](SparseTensor& t, u32arr a) {
                 if ((uint64_t)a.size() != t.indices.shape[0] * t.dim)
                     throw std::runtime_error("index shape mismatch");
                 std::copy(a.data(), a.data() + a.size(), t.indices());
             })
        .def("get_perm",
             [](SparseTensor& t, int i) {
                 u32arr out({(py::ssize_t)t.perms[i].shape[0]});
                 std::copy(t.perms[i](), t.perms[i](t.perms[i].shape[0]), out.mutable_data());
                 return out;
             })
        .def("get_values", [](SparseTensor& t) { return buffer_rows(t.values, t.values.shape[0], 1); });

    py::class_<ALS_Optimizer>(m, "ALS_Optimizer")
        .def("initialize_ground_truth_for_als", &ALS_Optimizer::initialize_ground_truth_for_als)
        .def("execute_ALS_rounds", &ALS_Optimizer::execute_ALS_rounds)
        .def("get_statistics_json", &ALS_Optimizer::get_statistics_json)
        .def("compute_exact_fit", &ALS_Optimizer::compute_exact_fit)
        .def("deinitialize", &ALS_Optimizer::deinitialize)
        .def("execute_ALS_step", &ALS_Optimizer::execute_ALS_step)
        .def("reset_counters", [](ALS_Optimizer& o) { o.nonzeros_iterated = 0.0; })
        .def_readonly("nonzeros_iterated", &ALS_Optimizer::nonzeros_iterated)
        .def("dedup", [](ALS_Optimizer& o, u32arr samples, f64arr weights, uint64_t mode) {
            uint64_t J = samples.shape(0), N = samples.shape(1);
            Buffer<uint32_t> s({J, N});
            Buffer<double> w({J});
            std::copy(samples.data(), samples.data() + J * N, s());
            std::copy(weights.data(), weights.data() + J, w());
            Buffer<uint32_t> sd;
            Buffer<double> wd;
            o.deduplicate_design_matrix(s, w, mode, sd, wd);
            uint64_t Ju = sd.shape[0];
            u32arr os({(py::ssize_t)Ju, (py::ssize_t)N});
            std::copy(sd(), sd(Ju * N), os.mutable_data());
            f64arr ow({(py::ssize_t)Ju});
            std::copy(wd(), wd(Ju), ow.mutable_data());
            return py::make_tuple(os, ow);
        });
    py::class_<ExactALS, ALS_Optimizer>(m, "ExactALS").def(py::init<SparseTensor&, LowRankTensor&>());
    py::class_<TensorStationary, ALS_Optimizer>(m, "TensorStationary")
        .def(py::init<SparseTensor&, LowRankTensor&, Sampler&>());
    py::class_<AccumulatorStationary, ALS_Optimizer>(m, "AccumulatorStationary")
        .def(py::init<SparseTensor&, LowRankTensor&, Sampler&>())
        // Sampled MTTKRP through the mode's sorted lookup (sort_lookup.hpp:238-375).
        .def("spmm", [](AccumulatorStationary& o, uint64_t mode, u32arr samples, f64arr design, uint64_t out_rows) {
            uint64_t Ju = samples.shape(0), N = samples.shape(1), R = design.shape(1);
            Buffer<uint32_t> s({Ju, N});
            Buffer<double> d({Ju, R});
            Buffer<double> out({out_rows, R});
            std::copy(samples.data(), samples.data() + Ju * N, s());
            std::copy(design.data(), design.data() + Ju * R, d());
            std::fill(out(), out(out_rows * R), 0.0);
            uint64_t found = o.lookups[mode]->csr_based_spmm(s, d, out);
            return py::make_tuple(buffer_rows(out, out_rows, R), found);
        });

    py::class_<StreamState>(m, "StreamState");
    py::class_<Sampler>(m, "Sampler")
        .def("reseed", &reseed)
        .def("update_sampler", &Sampler::update_sampler)
        .def("save_streams", &save_streams)
        .def("restore_streams", &restore_streams);
    py::class_<CP_ARLS_LEV, Sampler>(m, "CP_ARLS_LEV")
        .def(py::init<LowRankTensor&>())
        .def("draw", &arls_draw)
        .def("leverage_scores", [](CP_ARLS_LEV& s, int j) {
            DistMat1D& f = s.U[j];
            return buffer_rows(s.leverage_scores[j], f.true_row_count, 1);
        });
    py::class_<STS_CP, Sampler>(m, "STS_CP")
        .def(py::init<LowRankTensor&>())
        .def("draw", &sts_draw)
        .def("get_M", [](STS_CP& s) { return buffer_rows(s.M, s.N + 2, s.R2); });

    // PartitionTree::build_tree + PTSample on a given matrix (partition_tree.hpp:117-380),
    // starting from h = 1: returns the sampled rows and h * U[row].
    m.def("pt_sample", [](f64arr U, uint32_t F, f64arr scaled_h, f64arr draws) {
        uint64_t n = U.shape(0), R = U.shape(1), J = scaled_h.shape(0);
        Buffer<double> Ub({n, R});
        std::copy(U.data(), U.data() + n * R, Ub());
        PartitionTree tree((uint32_t)n, F, R);
        tree.build_tree(Ub);
        Buffer<double> h({J, R});
        Buffer<double> sh({J, R});
        std::fill(h(), h(J * R), 1.0);
        std::copy(scaled_h.data(), scaled_h.data() + J * R, sh());
        Buffer<uint32_t> samples({J, 1});
        Buffer<double> d({J});
        std::copy(draws.data(), draws.data() + J, d());
        ScratchBuffer scratch(F, J, R);
        tree.PTSample(Ub, h, sh, samples, d, scratch, 0);
        u32arr out({(py::ssize_t)J});
        std::copy(samples(), samples(J), out.mutable_data());
        return py::make_tuple(out, buffer_rows(h, J, R), buffer_rows(tree.G, tree.node_count, R * R));
    });
    m.def("pinv_square", [](f64arr M) {
        uint64_t R = M.shape(0);
        Buffer<double> a({R, R});
        Buffer<double> out({R, R});
        std::copy(M.data(), M.data() + R * R, a());
        std::fill(out(), out(R * R), 0.0);
        compute_pinv_square(a, out, R);
        return buffer_rows(out, R, R);
    });
}
