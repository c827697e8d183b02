// virtual_graph.cpp -- VirtualGraph / UMVirtualGraph of the C++ facade
// (reference src/virtual_graph.cpp:3-112, src/um_virtual_graph.cu:3-111).
//
// The constructor keeps the reference's observable behaviour: ids of a file without id 0 are shifted
// down by one in the Graph itself (src/virtual_graph.cpp:5-12) and in/out degrees are counted.
// MakeGraph() builds the device virtual graph (lossless, GPU segmented scan) and exports the host
// arrays in the reference layout for code that reads them (for instance a --debug CPU check).
#include <stdexcept>
#include <string>
#include <vector>

#include "eegraph.hpp"

namespace {

template <class G>
void shift_and_count(G& graph, uint*& inDeg, uint*& outDeg) {
    if (!graph.hasZeroID) {
        for (uint i = 0; i < graph.num_edges; ++i) {
            graph.edges[i].source -= 1;
            graph.edges[i].end -= 1;
        }
        // ids are now 0-based: a second VirtualGraph on the same Graph must not shift again
        graph.hasZeroID = true;
    }
    inDeg = new uint[graph.num_nodes]();
    outDeg = new uint[graph.num_nodes]();
    for (uint i = 0; i < graph.num_edges; ++i) {
        if (graph.edges[i].source >= graph.num_nodes) continue;
        outDeg[graph.edges[i].source]++;
        if (graph.edges[i].end >= graph.num_nodes) continue;
        inDeg[graph.edges[i].end]++;
    }
}

eeg_vgraph* build_from_edges(const Edge* edges, const uint* weights, uint n, uint m, unsigned K, uint32_t flags) {
    std::vector<uint32_t> s(m), d(m);
    for (uint i = 0; i < m; ++i) {
        s[i] = edges[i].source;
        d[i] = edges[i].end;
    }
    eeg_vgraph* vg = nullptr;
    if (eeg_vgraph_build_arrays(n, m, s.data(), d.data(), weights, K, flags, nullptr, &vg) != EEG_OK)
        throw std::runtime_error(std::string("virtual graph build failed: ") + eeg_last_error());
    return vg;
}

template <class VG>
void export_layout(VG& v, eeg_vgraph* dev, uint n, uint m) {
    eeg_vgraph_info info;
    eeg_vgraph_get_info(dev, &info);
    v.numParts = (decltype(v.numParts))info.num_parts;
    v.nodePointer = new uint[n ? n : 1];
    v.edgeList = new uint[2 * (size_t)m + n + 1];
    v.partNodePointer = new PartPointer[info.num_parts ? info.num_parts : 1];
    if (eeg_vgraph_export_reference_layout(dev, v.nodePointer, v.edgeList, (uint32_t*)v.partNodePointer) != EEG_OK)
        throw std::runtime_error(std::string("virtual graph export failed: ") + eeg_last_error());
}

}  // namespace

VirtualGraph::VirtualGraph(Graph& g, unsigned int K) : graph(&g), K_(K) { shift_and_count(g, inDegree, outDegree); }

VirtualGraph::~VirtualGraph() {
    delete[] edgeList;
    delete[] nodePointer;
    delete[] inDegree;
    delete[] outDegree;
    delete[] partNodePointer;
    eeg_vgraph_destroy(dev_);
}

void VirtualGraph::MakeGraph() {
    if (dev_) return;
    weights = graph->weights;
    if (weights.size() != graph->edges.size()) weights.assign(graph->edges.size(), 1u);
    dev_ = build_from_edges(graph->edges.data(), weights.data(), graph->num_nodes, graph->num_edges, K_, 0);
    export_layout(*this, dev_, graph->num_nodes, graph->num_edges);
}

UMVirtualGraph::UMVirtualGraph(UMGraph& g, unsigned int K) : graph(&g), K_(K) { shift_and_count(g, inDegree, outDegree); }

UMVirtualGraph::~UMVirtualGraph() {
    delete[] edgeList;
    delete[] nodePointer;
    delete[] inDegree;
    delete[] outDegree;
    delete[] partNodePointer;
    eeg_vgraph_destroy(dev_);
}

void UMVirtualGraph::MakeGraph() {
    if (dev_) return;
    dev_ = build_from_edges(graph->edges, graph->weights, graph->num_nodes, graph->num_edges, K_, EEG_VG_MANAGED);
    export_layout(*this, dev_, graph->num_nodes, graph->num_edges);
}
