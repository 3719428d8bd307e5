// Checker build of the reference's own vertex-coloring algorithms — TEST INFRASTRUCTURE
// ONLY. Compiled by `make -C oracle ref` from the reference tree (GraphColoring/mcs.cpp,
// gready.cpp, ColoringAlgorithms.cpp, with ref_shim/ standing in for the MeshFrame
// headers that Graph.h includes) into oracle/_ref/libcolor_ref.so. The tests compare the
// library's and the oracle's MCS / OrderedGreedy with it on arbitrary vertex graphs.
#include <cstdint>
#include <vector>

#include "GraphColoring/gready.h"
#include "GraphColoring/mcs.h"

namespace {
// access to the categories the tool writes
template <typename Alg>
struct WithCategories : Alg {
    using Alg::Alg;
    const std::vector<std::vector<int>>& cats() const { return this->categories; }
};
}  // namespace

// The GraphColoring tool's pipeline (GraphColoring.cpp:170-189): color, categories,
// optional balancing; colors and the categories' vertex order out.
extern "C" int32_t ref_color_tool(int32_t algo, int32_t balance, float goal, int32_t nv, const int64_t* ofs,
                                  const int32_t* adj, int32_t* colors, int32_t* order) {
    std::vector<std::vector<int>> g(static_cast<size_t>(nv));
    for (int32_t v = 0; v < nv; ++v) g[size_t(v)].assign(adj + ofs[v], adj + ofs[v + 1]);
    auto run = [&](auto& m) {
        m.color();
        m.convertToColoredCategories();
        if (balance) m.balanceColoredCategories(goal);
        if (!m.is_valid()) return int32_t(-1);
        int32_t n = 0, k = 0;
        for (int32_t v = 0; v < nv; ++v) {
            colors[v] = m.get_color(v);
            n = colors[v] + 1 > n ? colors[v] + 1 : n;
        }
        for (const auto& c : m.cats())
            for (int v : c) order[k++] = v;
        return n;
    };
    if (algo == 0) {
        WithCategories<GAIA::GraphColoring::Mcs> m(g);
        return run(m);
    }
    WithCategories<GAIA::GraphColoring::OrderedGreedy> m(g);
    return run(m);
}

// algo 0 = MCS, 1 = OrderedGreedy; the graph as CSR (ofs has nv + 1 entries). Returns the
// number of colors, or -1 if the reference reports an invalid coloring.
extern "C" int32_t ref_color(int32_t algo, int32_t nv, const int64_t* ofs, const int32_t* adj, int32_t* colors) {
    std::vector<std::vector<int>> g(static_cast<size_t>(nv));
    for (int32_t v = 0; v < nv; ++v) g[size_t(v)].assign(adj + ofs[v], adj + ofs[v + 1]);
    std::vector<int> c;
    if (algo == 0) {
        GAIA::GraphColoring::Mcs m(g);
        c = m.color();
        if (!m.is_valid()) return -1;
    } else {
        GAIA::GraphColoring::OrderedGreedy m(g);
        c = m.color();
        if (!m.is_valid()) return -1;
    }
    int32_t n = 0;
    for (int32_t v = 0; v < nv; ++v) {
        colors[v] = c[size_t(v)];
        n = colors[v] + 1 > n ? colors[v] + 1 : n;
    }
    return n;
}
