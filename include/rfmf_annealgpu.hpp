// rfmf_annealgpu.hpp -- gpu3::annealGpu on top of librfmf.so.
//
// Drop-in definition of the reference's solver entry point
//   void gpu3::annealGpu(const anneallib::AnnealCsr&, int64_t maxWeightedDeg,
//                        const std::vector<std::vector<int8_t>>& initialSpins,
//                        const std::vector<double>& t0s,
//                        const std::vector<size_t>& phases,
//                        const std::vector<uint64_t>& iters,
//                        const std::vector<uint64_t>& solverSeeds,
//                        const LaunchConfig& cfg,
//                        std::vector<std::vector<int8_t>>& endSpins,
//                        std::vector<std::vector<int8_t>>& bestSpins,
//                        float* kernelMs,
//                        std::vector<int64_t>* kernelBestVals,
//                        std::vector<int64_t>* kernelFinalVals)
// declared at src/anneal_gpu.cuh:76-88 (defined by the reference at
// src/anneal_kernels.cu:835-884).  Include it in ONE translation unit AFTER
// the reference's own "anneal_gpu.cuh" (which declares the signature and
// LaunchConfig), in place of compiling src/anneal_kernels.cu, and link
// against librfmf.so.  main.cu and the reference's host code stay unchanged.
//
// Behaviour mirrors the reference: synchronous, outputs resized and filled,
// *kernelMs is the device time of the annealing launch(es), and errors are
// fatal (message on stderr, std::exit(EXIT_FAILURE)) exactly where the
// reference exits; the C ABI underneath returns status codes instead.
#ifndef RFMF_ANNEALGPU_HPP
#define RFMF_ANNEALGPU_HPP

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rfmf.h"

namespace gpu3 {

namespace rfmf_shim {
inline void check(int rc, const char* what) {
    if (rc != RFMF_OK) {
        std::fprintf(stderr, "Error: %s failed: %s\n", what, rfmf_last_error());
        std::exit(EXIT_FAILURE);
    }
}
}  // namespace rfmf_shim

void annealGpu(const anneallib::AnnealCsr& ig, int64_t maxWeightedDeg,
               const std::vector<std::vector<int8_t>>& initialSpins,
               const std::vector<double>& t0s, const std::vector<size_t>& phases,
               const std::vector<uint64_t>& iters, const std::vector<uint64_t>& solverSeeds,
               const LaunchConfig& cfg, std::vector<std::vector<int8_t>>& endSpins,
               std::vector<std::vector<int8_t>>& bestSpins, float* kernelMs,
               std::vector<int64_t>* kernelBestVals, std::vector<int64_t>* kernelFinalVals) {
    using rfmf_shim::check;
    const size_t C = t0s.size();
    if (C == 0 || solverSeeds.size() != C || initialSpins.size() != C) {
        std::fprintf(stderr,
                     "Error: annealGpu needs non-empty, equal-length t0s (%zu), "
                     "solverSeeds (%zu) and initialSpins (%zu).\n",
                     t0s.size(), solverSeeds.size(), initialSpins.size());
        std::exit(EXIT_FAILURE);
    }
    // Flatten the frozen CSR (dense ids, rows ascending).
    const int64_t n = static_cast<int64_t>(ig.numVertices());
    std::vector<uint32_t> off(static_cast<size_t>(n) + 1, 0);
    std::vector<int32_t> col, w;
    col.reserve(ig.numEdges() * 2);
    w.reserve(ig.numEdges() * 2);
    for (int64_t v = 0; v < n; ++v) {
        auto nb = ig.neighbors(v);
        for (uint32_t i = 0; i < nb.size(); ++i) {
            col.push_back(nb.to[i]);
            w.push_back(static_cast<int32_t>(nb.weight[i]));
        }
        off[static_cast<size_t>(v) + 1] = static_cast<uint32_t>(col.size());
    }
    std::vector<int8_t> init(C * static_cast<size_t>(n));
    for (size_t c = 0; c < C; ++c) {
        if (static_cast<int64_t>(initialSpins[c].size()) != n) {
            std::fprintf(stderr, "Error: initialSpins[%zu] has %zu entries, graph has %lld.\n", c,
                         initialSpins[c].size(), static_cast<long long>(n));
            std::exit(EXIT_FAILURE);
        }
        std::copy(initialSpins[c].begin(), initialSpins[c].end(), init.begin() + c * n);
    }
    std::vector<uint64_t> ph(phases.begin(), phases.end());

    rfmf_context* ctx = nullptr;
    check(rfmf_context_create(cfg.device, &ctx), "rfmf_context_create");
    rfmf_graph* g = nullptr;
    check(rfmf_graph_create(ctx, n, off.data(), col.data(), w.data(), &g), "rfmf_graph_create");
    rfmf_launch_config lc{};
    lc.corr = static_cast<int>(cfg.corr);
    lc.device = cfg.device;
    lc.s_width = cfg.sWidth;
    std::vector<int8_t> endFlat(init.size()), bestFlat(init.size());
    std::vector<int64_t> bv(C), fv(C);
    float ms = 0.0f;
    check(rfmf_anneal(ctx, g, maxWeightedDeg, static_cast<int64_t>(C), init.data(), t0s.data(),
                      static_cast<int64_t>(ph.size()), ph.data(), iters.data(),
                      solverSeeds.data(), &lc, endFlat.data(), bestFlat.data(), &ms, bv.data(),
                      fv.data()),
          "rfmf_anneal");
    rfmf_graph_destroy(g);
    rfmf_context_destroy(ctx);

    endSpins.resize(C);
    bestSpins.resize(C);
    for (size_t c = 0; c < C; ++c) {
        endSpins[c].assign(endFlat.begin() + c * n, endFlat.begin() + (c + 1) * n);
        bestSpins[c].assign(bestFlat.begin() + c * n, bestFlat.begin() + (c + 1) * n);
    }
    if (kernelMs) *kernelMs = ms;
    if (kernelBestVals) *kernelBestVals = bv;
    if (kernelFinalVals) *kernelFinalVals = fv;
}

}  // namespace gpu3

#endif  // RFMF_ANNEALGPU_HPP
