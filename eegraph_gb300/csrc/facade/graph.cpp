// graph.cpp -- Graph / UMGraph / VertexSubgraph of the C++ facade (reference src/graph.cpp:1-203,
// src/um_graph.cu:1-122). Parsing is done by eeg_graph_load (same rules as the reference,
// multi-threaded); these classes keep the reference's public fields and console output.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <vector>

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

// ------------------------------------------------------------------ VertexSubgraph
VertexSubgraph::VertexSubgraph(Graph& graph, std::string graphFilePath, bool isWeighted)
    : Graph(graphFilePath, isWeighted), parentGraph(&graph) {}

VertexSubgraph::~VertexSubgraph() { delete[] selected; }

namespace {

// One C-library draw, or two combined where the ids reach past RAND_MAX (every id stays reachable).
uint draw(uint range) {
    if ((unsigned long long)range <= (unsigned long long)RAND_MAX + 1ull) return (uint)rand() % range;
    const unsigned long long hi = (unsigned long long)rand(), lo = (unsigned long long)rand();
    return (uint)((hi * ((unsigned long long)RAND_MAX + 1ull) + lo) % range);
}

// pct of the n vertices: the source, then rand() draws seeded by `seed`, the first half of them from
// the lowest fifth of the ids. Returns the number kept; `selected` must hold n zeroed flags.
// The reference's loop (src/graph.cpp:148-164) never ends once the first half needs more distinct ids
// than the lowest fifth holds (pct above about 0.4); here the draws move to the whole range when the
// lowest fifth is used up, so every pct in [0, 1] ends, and the draws are the reference's whenever its
// loop ends.
uint select_vertices(uint n, float pct, int sourceNode, time_t seed, bool* selected) {
    const float p = std::min(1.0f, std::max(0.0f, pct));
    const uint target = (uint)(p * n);  // a float product, as the reference's `pct * num_nodes`
    uint count = 0;
    const uint low = n / 5 ? n / 5 : n;
    uint low_taken = 0;  // selected ids below `low`
    if (n > 0 && sourceNode >= 0 && (uint)sourceNode < n) {
        selected[sourceNode] = true;
        count = 1;
        low_taken = (uint)sourceNode < low ? 1 : 0;
    }
    srand((unsigned)seed);
    while (count < target) {
        const bool from_low = count < target / 2 && low_taken < low;
        const uint v = draw(from_low ? low : n);
        if (!selected[v]) {
            selected[v] = true;
            ++count;
            if (v < low) ++low_taken;
        }
    }
    return target;
}

void print_subgraph(float ms, uint kept, uint n, uint m) {
    std::cout << "Done generating subgraph.\n";
    std::cout << "Subgraph generated in " << ms << " (ms)" << std::endl;
    std::cout << "Subgraph number of nodes = " << kept << std::endl;
    std::cout << "Virtual graph assumed number of nodes = " << n << std::endl;
    std::cout << "Subgraph number of edges = " << m << std::endl;
}

}  // namespace

void VertexSubgraph::MakeSubgraph(float pct_, int sourceNode, time_t seed) {
    graphLoaded = parentGraph->graphLoaded;
    pct = pct_;
    if (!graphLoaded) {
        std::cout << "Graph has not been loaded" << std::endl;
        return;
    }
    const uint n = parentGraph->num_nodes;
    num_nodes = n;
    Timer overhead;
    overhead.Start();
    delete[] selected;
    selected = new bool[n ? n : 1]();
    subgraph_num_nodes = select_vertices(n, pct, sourceNode, seed, selected);
    edges.clear();
    weights.clear();
    hasZeroID = false;
    for (size_t i = 0; i < parentGraph->edges.size(); ++i) {
        const Edge e = parentGraph->edges[i];
        if (e.source < n && e.end < n && selected[e.source] && selected[e.end]) {
            if (e.source == 0 || e.end == 0) hasZeroID = true;
            if (isWeighted) weights.push_back(i < parentGraph->weights.size() ? parentGraph->weights[i] : 1u);
            edges.push_back(e);
        }
    }
    num_edges = (uint)edges.size();
    print_subgraph(overhead.Finish(), subgraph_num_nodes, num_nodes, num_edges);
}

// ------------------------------------------------------------------ UMVertexSubgraph
UMVertexSubgraph::UMVertexSubgraph(UMGraph& graph, std::string graphFilePath, bool isWeighted)
    : UMGraph(graphFilePath, isWeighted), parentGraph(&graph) {}

UMVertexSubgraph::~UMVertexSubgraph() { delete[] selected; }

void UMVertexSubgraph::MakeSubgraph(float pct_, int sourceNode, time_t seed) {
    graphLoaded = parentGraph->graphLoaded;
    pct = pct_;
    if (!graphLoaded) {
        std::cout << "Graph has not been loaded" << std::endl;
        return;
    }
    const uint n = parentGraph->num_nodes;
    num_nodes = n;
    Timer overhead;
    overhead.Start();
    delete[] selected;
    selected = new bool[n ? n : 1]();
    subgraph_num_nodes = select_vertices(n, pct, sourceNode, seed, selected);
    std::vector<Edge> ke;
    std::vector<uint> kw;
    hasZeroID = false;
    for (uint i = 0; i < parentGraph->num_edges; ++i) {
        const Edge e = parentGraph->edges[i];
        if (e.source < n && e.end < n && selected[e.source] && selected[e.end]) {
            if (e.source == 0 || e.end == 0) hasZeroID = true;
            ke.push_back(e);
            kw.push_back(parentGraph->weights ? parentGraph->weights[i] : 1u);
        }
    }
    eeg_managed_free(edges);
    eeg_managed_free(weights);
    edges = nullptr;
    weights = nullptr;
    if (eeg_managed_alloc(sizeof(Edge) * (ke.empty() ? 1 : ke.size()), (void**)&edges) != EEG_OK ||
        eeg_managed_alloc(sizeof(uint) * (kw.empty() ? 1 : kw.size()), (void**)&weights) != EEG_OK)
        throw std::runtime_error(std::string("UMVertexSubgraph: ") + eeg_last_error());
    std::copy(ke.begin(), ke.end(), edges);
    std::copy(kw.begin(), kw.end(), weights);
    num_edges = (uint)ke.size();
    print_subgraph(overhead.Finish(), subgraph_num_nodes, num_nodes, num_edges);
}
