// main.cpp -- the per-algorithm executables bfs-main, sssp-main, sswp-main, cc-main and pr-main
// (reference src/{bfs,sssp,sswp,cc,pr}_main.cu). One program; the algorithm is taken from the name it
// is started under. Flags are the reference's (--input --source --variant --um --debug ...).
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>

#include "eegraph.hpp"

int main(int argc, char** argv) {
    std::string name = argv[0];
    const size_t slash = name.find_last_of('/');
    if (slash != std::string::npos) name = name.substr(slash + 1);
    const std::string algo = name.substr(0, name.find('-'));
    if (algo != "bfs" && algo != "sssp" && algo != "sswp" && algo != "cc" && algo != "pr") {
        std::cerr << "unknown algorithm in program name: " << name << "\n";
        return 2;
    }
    ArgumentParser arguments(argc, argv, true, false);
    try {
        if (arguments.unifiedMem) {
            UMGraph graph(arguments.input, true);
            graph.ReadGraph();
            if (graph.num_nodes < 1) {
                std::cout << "Graph file not read correctly" << std::endl;
                return -1;
            }
            if (algo == "bfs") eegraph_bfs_um(arguments, graph);
            else if (algo == "sssp") eegraph_sssp_um(arguments, graph);
            else if (algo == "sswp") eegraph_sswp_um(arguments, graph);
            else if (algo == "cc") eegraph_cc_um(arguments, graph);
            else eegraph_pr_um(arguments, graph);
        } else {
            Graph graph(arguments.input, true);
            graph.ReadGraph();
            if (graph.num_nodes < 1) {
                std::cout << "Graph file not read correctly" << std::endl;
                return -1;
            }
            if (algo == "bfs") eegraph_bfs(arguments, graph);
            else if (algo == "sssp") eegraph_sssp(arguments, graph);
            else if (algo == "sswp") eegraph_sswp(arguments, graph);
            else if (algo == "cc") eegraph_cc(arguments, graph);
            else eegraph_pr(arguments, graph);
        }
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 1;
    }
    return 0;
}
