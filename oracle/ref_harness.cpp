// ref_harness.cpp -- C entry points onto the reference's OWN host code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file together
// with the reference's host sources where they lie (src/host_common.cpp,
// src/max_cut.cpp, src/read_gset.cpp, src/graph.cpp and the header-only
// src/philox.cuh, src/rng.hpp, src/immutable_graph.hpp) into
// oracle/_ref/libref_host.so.  Tests use it, where it exists, to check the
// oracle's restatement against the reference and to generate the golden
// fixtures under tests/golden/.  Nothing here is shipped or timed.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "host_common.h"
#include "immutable_graph.hpp"
#include "max_cut.hpp"
#include "philox.cuh"
#include "read_gset.hpp"
#include "rng.hpp"

extern "C" {

// src/philox.cuh:89-119
void ref_philox_block(uint64_t seed, uint64_t step, uint64_t block, uint32_t out[4]) {
    const gpu3::Philox4 r = gpu3::philox4x32_10(gpu3::gumbelBlockCounter(step, block),
                                                gpu3::philoxKeyFromSeed(seed));
    for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

// src/philox.cuh:52-58, 121-126
int32_t ref_gumbel_field(uint64_t seed, uint64_t step, uint64_t block, uint32_t j) {
    const gpu3::Philox4 r = gpu3::philox4x32_10(gpu3::gumbelBlockCounter(step, block),
                                                gpu3::philoxKeyFromSeed(seed));
    return gpu3::gumbelFromBitsG(gpu3::gumbelBitsFromBlock(r, j));
}

int32_t ref_gumbel(uint32_t r11) { return gpu3::gumbelFromBitsG(r11); }

uint64_t ref_pack_score_id(int32_t score, int32_t id) { return gpu3::packScoreId(score, id); }

// src/host_common.h:73-76
int32_t ref_beta_fixed(uint64_t step, double t0) { return betaFixedForStep(step, t0); }

// src/host_common.cpp:238-294.  Returns the run count; fills up to cap runs.
int64_t ref_beta_tables(const double* t0s, int64_t C, int64_t total_steps,
                        int64_t* run_end, int32_t* run_val, int64_t* chain_off,
                        int64_t cap) {
    std::vector<double> t(t0s, t0s + C);
    const BetaRunTables bt = buildBetaRunTables(t, total_steps);
    const int64_t runs = static_cast<int64_t>(bt.runEnd.size());
    for (int64_t i = 0; i < runs && i < cap; ++i) {
        run_end[i] = bt.runEnd[i];
        run_val[i] = bt.runVal[i];
    }
    for (int64_t c = 0; c < C; ++c) chain_off[c] = bt.chainRunOff[c];
    return runs;
}

// src/host_common.cpp:296-312
int ref_score_safe_int32(int64_t total_steps, double t0, int64_t B) {
    return annealScoreSafeInt32(total_steps, t0, B) ? 1 : 0;
}

// src/rng.hpp + the draw loop of src/host_common.cpp:40-45
void ref_initial_spins(uint64_t seed, int64_t n, int8_t* out) {
    anneallib::Rng rng(seed);
    for (int64_t i = 0; i < n; ++i) out[i] = static_cast<int8_t>(rng.bits(1) ? 1 : -1);
}

// Graph file -> Graph -> degree-0 removal -> AnnealCsr, as setupSolver does
// (src/host_common.cpp:333-348).
struct RefGraph {
    anneallib::AnnealCsr csr;
    anneallib::ReadStats stats;
};

void* ref_gset_load(const char* path) {
    anneallib::Graph g;
    auto* h = new RefGraph();
    if (!anneallib::read_instance_from_file(path, g, &h->stats, 0.0)) {
        delete h;
        return nullptr;
    }
    removeDegreeZeroVertices(g);
    h->csr = anneallib::AnnealCsr(g);
    return h;
}

double ref_gset_scale(void* h) { return static_cast<RefGraph*>(h)->stats.scale; }
int64_t ref_gset_zero_dropped(void* h) { return static_cast<RefGraph*>(h)->stats.zeroDropped; }

int64_t ref_gset_n(void* h) { return static_cast<int64_t>(static_cast<RefGraph*>(h)->csr.numVertices()); }
int64_t ref_gset_m(void* h) { return static_cast<int64_t>(static_cast<RefGraph*>(h)->csr.numEdges()); }

void ref_gset_copy(void* hv, uint32_t* offsets, int32_t* col, int32_t* w) {
    const auto& csr = static_cast<RefGraph*>(hv)->csr;
    const int64_t n = static_cast<int64_t>(csr.numVertices());
    uint32_t pos = 0;
    offsets[0] = 0;
    for (int64_t v = 0; v < n; ++v) {
        auto nb = csr.neighbors(v);
        for (uint32_t i = 0; i < nb.size(); ++i) {
            col[pos] = nb.to[i];
            w[pos] = nb.weight[i];
            ++pos;
        }
        offsets[v + 1] = pos;
    }
}

// src/max_cut.cpp:5-15 and src/host_common.cpp:314-325 on the loaded graph.
int64_t ref_gset_cut(void* hv, const int8_t* spin) {
    const auto& csr = static_cast<RefGraph*>(hv)->csr;
    std::vector<int8_t> s(spin, spin + csr.numVertices());
    return anneallib::solver::cutValueCsr(csr, s);
}

int64_t ref_gset_max_weighted_degree(void* hv) {
    return maxWeightedDegree(static_cast<RefGraph*>(hv)->csr);
}

void ref_gset_free(void* h) { delete static_cast<RefGraph*>(h); }

}  // extern "C"
