// graph_info.cpp -- graph-info-main, the reference's graph_info program (src/graph_info.cpp): reads the
// graph given with --input and prints its largest out-degree and the average out-degree of the first
// 20 % of the vertex ids and of the remaining 80 % (R-MAT-like generators put the hubs at low ids).
// Unlike the reference, every vertex's degree starts at zero (it left those without out-edges unset).
#include <algorithm>
#include <iostream>
#include <vector>

#include "eegraph.hpp"

int main(int argc, char** argv) {
    ArgumentParser arguments(argc, argv, true, false);
    Graph graph(arguments.input, true);
    graph.ReadGraph();
    const uint n = graph.num_nodes;
    std::vector<uint> degree(n ? n : 1, 0u);
    uint max = 0;
    for (const Edge& e : graph.edges)
        if (e.source < n) max = std::max(max, ++degree[e.source]);
    std::cout << "Max degree: " << max << std::endl;
    const uint cut = (uint)(.20 * n);
    double sum = 0;
    for (uint j = 0; j < cut; ++j) sum += degree[j];
    std::cout << "Avg Degree First 20 percent of Vertices: " << (cut ? (float)(sum / cut) : 0.f) << std::endl;
    sum = 0;
    for (uint j = cut; j < n; ++j) sum += degree[j];
    std::cout << "Avg Degree Remaining 80 percent of Vertices: " << (n > cut ? (float)(sum / (n - cut)) : 0.f)
              << std::endl;
    return 0;
}
