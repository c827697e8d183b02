// graph.cpp -- Graph / UMGraph of the C++ facade (reference src/graph.cpp:1-120, src/um_graph.cu:1-122).
// Parsing is done by eeg_graph_load (same rules as the reference, multi-threaded); these classes
// keep the reference's public fields and console output.
#include <cstring>
#include <iostream>
#include <stdexcept>

#include "eegraph.hpp"

namespace {

std::string ext_of(const std::string& f) {
    const size_t dot = f.find_last_of('.');
    return dot == std::string::npos ? std::string() : f.substr(dot + 1);
}

bool known_ext(const std::string& e) {
    return e == "bcsr" || e == "bwcsr" || e == "edges" || e == "el" || e == "wel" || e == "txt" || e == "edgelist";
}

}  // namespace

Graph::Graph(std::string path, bool weighted)
    : graphFilePath(std::move(path)), isWeighted(weighted), hasZeroID(false), graphLoaded(false) {}

std::string Graph::getFileExtension(std::string fileName) { return ext_of(fileName); }

void Graph::ReadGraph() {
    std::cout << "Reading the input graph from the following file:\n>> " << graphFilePath << std::endl;
    graphFormat = getFileExtension(graphFilePath);
    if (!known_ext(graphFormat)) {
        std::cout << "Graph file type not recognized" << std::endl;
    } else {
        eeg_graph* g = nullptr;
        // The reference loader always records weights (1 when absent); the text path keeps them only
        // when isWeighted, like src/graph.cpp:87-93.
        eeg_status s = eeg_graph_load(graphFilePath.c_str(), isWeighted ? 1 : 0, 0, &g);
        if (s != EEG_OK) {
            std::cout << "Error reading graph: " << eeg_last_error() << std::endl;
        } else {
            eeg_graph_view v;
            eeg_graph_view_get(g, &v);
            edges.resize(v.num_edges);
            for (uint64_t e = 0; e < v.num_edges; ++e) edges[e] = Edge{v.src[e], v.dst[e]};
            weights.clear();
            if (v.weight) weights.assign(v.weight, v.weight + v.num_edges);
            num_nodes = v.num_nodes;
            num_edges = (uint)v.num_edges;
            hasZeroID = v.has_zero_id != 0;
            graphLoaded = true;
            eeg_graph_destroy(g);
        }
    }
    std::cout << "Done reading.\n";
    std::cout << "Number of nodes = " << num_nodes << std::endl;
    std::cout << "Number of edges = " << num_edges << std::endl;
}

UMGraph::UMGraph(std::string path, bool weighted)
    : graphFilePath(std::move(path)), isWeighted(weighted), hasZeroID(false), graphLoaded(false) {}

UMGraph::~UMGraph() {
    eeg_managed_free(edges);
    eeg_managed_free(weights);
}

std::string UMGraph::getFileExtension(std::string fileName) { return ext_of(fileName); }

void UMGraph::ReadGraph() {
    std::cout << "Reading the input graph from the following file:\n>> " << graphFilePath << std::endl;
    graphFormat = getFileExtension(graphFilePath);
    if (!known_ext(graphFormat)) {
        std::cout << "Graph file type not recognized" << std::endl;
    } else {
        eeg_graph* g = nullptr;
        eeg_status s = eeg_graph_load(graphFilePath.c_str(), 1, 0, &g);
        if (s != EEG_OK) {
            std::cout << "Error reading graph: " << eeg_last_error() << std::endl;
        } else {
            eeg_graph_view v;
            eeg_graph_view_get(g, &v);
            eeg_managed_free(edges);
            eeg_managed_free(weights);
            edges = nullptr;
            weights = nullptr;
            if (eeg_managed_alloc(sizeof(Edge) * (v.num_edges ? v.num_edges : 1), (void**)&edges) != EEG_OK ||
                eeg_managed_alloc(sizeof(uint) * (v.num_edges ? v.num_edges : 1), (void**)&weights) != EEG_OK) {
                eeg_graph_destroy(g);
                throw std::runtime_error(std::string("managed allocation failed: ") + eeg_last_error());
            }
            for (uint64_t e = 0; e < v.num_edges; ++e) {
                edges[e] = Edge{v.src[e], v.dst[e]};
                weights[e] = v.weight ? v.weight[e] : 1u;
            }
            num_nodes = v.num_nodes;
            num_edges = (uint)v.num_edges;
            hasZeroID = v.has_zero_id != 0;
            graphLoaded = true;
            eeg_graph_destroy(g);
        }
    }
    std::cout << "Done reading.\n";
    std::cout << "Number of nodes = " << num_nodes << std::endl;
    std::cout << "Number of edges = " << num_edges << std::endl;
}
