// eegraph.hpp -- C++ facade with the reference's types and entry points, built on include/eegraph_c.h.
//
// Source-compatible replacements for (rwatling/EEGraph paths):
//   include/globals.hpp:30-57          Part_Size, DIST_INFINITY, Variant, Edge, PartPointer, Result
//   include/graph.hpp:28-50            class Graph          (src/graph.cpp)
//   include/virtual_graph.hpp:8-26     class VirtualGraph   (src/virtual_graph.cpp)
//   include/um_graph.cuh:28-50         class UMGraph        (src/um_graph.cu)
//   include/um_virtual_graph.cuh:7-23  class UMVirtualGraph (src/um_virtual_graph.cu)
//   include/argument_parsing.hpp:6-49  class ArgumentParser (src/argument_parsing.cpp)
//   include/utilities.hpp:8-16         namespace utilities  (src/utilities.cpp)
//   include/timer.hpp                  class Timer          (src/timer.cpp)
//   include/eegraph.cuh:21-39          eegraph_{bfs,cc,pr,sswp,sssp}[_um]
// Differences a caller can see are listed beside each declaration.
#ifndef EEGRAPH_HPP
#define EEGRAPH_HPP

#include <sys/time.h>

#include <climits>
#include <ctime>
#include <string>
#include <vector>

#include "eegraph_c.h"

typedef unsigned int uint;

// Default Tigr part size K; here a run-time choice (4, 8 or 16), --k on the command line.
const unsigned int Part_Size = 8;
const unsigned int DIST_INFINITY = UINT_MAX - 1;

enum Variant : unsigned char {
    ASYNC_PUSH_TD,
    ASYNC_PUSH_DD,
    SYNC_PUSH_TD,
    SYNC_PUSH_DD,
};

struct Edge {
    unsigned int source;
    unsigned int end;
};

struct PartPointer {
    unsigned int node;
    unsigned int part;
};

// time (ms, total GPU activity), energy (joules; negative when NVML is unavailable) and the
// per-iteration active-vertex counts, as in the reference; plus run statistics.
struct Result {
    float time = 0.f;
    double energy = 0.0;
    std::vector<unsigned int> sumLabelsVec;
    float processingTime = 0.f;   // device time of the traversal (CUDA events)
    unsigned int iterations = 0;
    double gteps = 0.0;
    double algorithmicBytes = 0.0;
    unsigned long long reachedVertices = 0, reachedEdges = 0;
};

class Timer {
   public:
    void Start() { gettimeofday(&StartingTime, nullptr); }
    float Finish() {
        timeval now, el;
        gettimeofday(&now, nullptr);
        timersub(&now, &StartingTime, &el);
        return el.tv_sec * 1000.0f + el.tv_usec / 1000.0f;
    }

   private:
    timeval StartingTime{};
};

// Host edge list. ReadGraph() keeps the reference's parsing rules and console messages.
class Graph {
   public:
    std::string graphFilePath;
    std::string graphFormat;
    bool isWeighted;
    bool hasZeroID;
    bool graphLoaded;
    uint num_nodes = 0;
    uint num_edges = 0;
    std::vector<Edge> edges;
    std::vector<uint> weights;

    Graph(std::string graphFilePath, bool isWeighted);
    void ReadGraph();
    std::string getFileExtension(std::string fileName);
};

// Vertex-induced subgraph for experiments (reference include/graph.hpp:52-63, src/graph.cpp:122-203):
// MakeSubgraph keeps pct of the parent's vertices -- the source, then vertices drawn with the C library's
// rand() seeded by `seed`, the first half of the draws from the lowest fifth of the ids -- and the edges
// whose both ends are kept. Ids are not renumbered (num_nodes stays the parent's, as the reference's
// "Virtual graph assumed number of nodes" line says). The same seed on the same C library gives the same
// subgraph. Unlike the reference it also works for graphs under five vertices and stops at 100 %.
class VertexSubgraph : public Graph {
   public:
    Graph* parentGraph;
    float pct = 0.f;
    bool* selected = nullptr;
    uint subgraph_num_nodes = 0;  // kept vertices (to pass into VirtualGraph)

    VertexSubgraph(Graph& graph, std::string graphFilePath, bool isWeighted);
    ~VertexSubgraph();
    VertexSubgraph(const VertexSubgraph&) = delete;
    VertexSubgraph& operator=(const VertexSubgraph&) = delete;
    void MakeSubgraph(float pct, int sourceNode, time_t seed);
};

// Managed-memory twin: edges/weights live in cudaMallocManaged memory.
class UMGraph {
   public:
    std::string graphFilePath;
    std::string graphFormat;
    bool isWeighted;
    bool hasZeroID;
    bool graphLoaded;
    uint num_nodes = 0;
    uint num_edges = 0;
    Edge* edges = nullptr;
    uint* weights = nullptr;

    UMGraph(std::string graphFilePath, bool isWeighted);
    ~UMGraph();
    void ReadGraph();
    std::string getFileExtension(std::string fileName);
};

// Managed-memory twin of VertexSubgraph (reference include/um_graph.cuh:52-63, src/um_graph.cu:124-200):
// the same selection; the kept edges and weights go to cudaMallocManaged arrays.
class UMVertexSubgraph : public UMGraph {
   public:
    UMGraph* parentGraph;
    float pct = 0.f;
    bool* selected = nullptr;
    uint subgraph_num_nodes = 0;

    UMVertexSubgraph(UMGraph& graph, std::string graphFilePath, bool isWeighted);
    ~UMVertexSubgraph();
    UMVertexSubgraph(const UMVertexSubgraph&) = delete;
    UMVertexSubgraph& operator=(const UMVertexSubgraph&) = delete;
    void MakeSubgraph(float pct, int sourceNode, time_t seed);
};

// K-bounded virtual graph. The constructor shifts 1-based ids down by one in the Graph it is
// given and counts degrees, as the reference's does. MakeGraph() builds the lossless virtual graph
// on the GPU and fills the public host arrays in the reference layout (nodePointer, edgeList =
// [deg,(t,w)...] per vertex, partNodePointer); numParts = sum ceil(outDegree/K).
class VirtualGraph {
   public:
    Graph* graph;
    uint* edgeList = nullptr;
    uint* nodePointer = nullptr;
    uint* inDegree = nullptr;
    uint* outDegree = nullptr;
    unsigned int numParts = 0;
    PartPointer* partNodePointer = nullptr;
    std::vector<uint> weights;

    explicit VirtualGraph(Graph& graph, unsigned int K = Part_Size);
    ~VirtualGraph();
    VirtualGraph(const VirtualGraph&) = delete;
    VirtualGraph& operator=(const VirtualGraph&) = delete;
    void MakeGraph();
    eeg_vgraph* device() const { return dev_; }  // device handle (valid after MakeGraph)

   private:
    unsigned int K_;
    eeg_vgraph* dev_ = nullptr;
};

class UMVirtualGraph {
   public:
    UMGraph* graph;
    uint* edgeList = nullptr;
    uint* nodePointer = nullptr;
    uint* inDegree = nullptr;
    uint* outDegree = nullptr;
    long long numParts = 0;
    PartPointer* partNodePointer = nullptr;

    explicit UMVirtualGraph(UMGraph& graph, unsigned int K = Part_Size);
    ~UMVirtualGraph();
    UMVirtualGraph(const UMVirtualGraph&) = delete;
    UMVirtualGraph& operator=(const UMVirtualGraph&) = delete;
    void MakeGraph();
    eeg_vgraph* device() const { return dev_; }

   private:
    unsigned int K_;
    eeg_vgraph* dev_ = nullptr;
};

// Command line: the reference's flags (--input --output --efile --estats --source --device --iteration
// --debug --activity --variant --energy --um --accuracy) with the same defaults and the same
// behaviour on errors (help text, exit(0)), plus --k {4,8,16}, --tolerance (PageRank L1 bound),
// --timeout (ms, device waits), --blocks-per-sm, --delta (bucketed SSSP/SSWP rounds),
// --cc-components (CC as connected components) and --stream-budget (MiB: keep the graph in host memory
// and stream each round's active subgraph through device buffers of that size, Subway's model;
// BFS/SSSP/SSWP/CC).
class ArgumentParser {
   public:
    int argc;
    char** argv;
    bool canHaveSource;
    bool canHaveItrs;
    bool hasInput = false;
    bool hasSourceNode = false;
    bool hasOutput = false;
    bool hasDeviceID = false;
    bool hasNumberOfItrs = false;
    bool hasEnergyFile = false;
    bool hasEnergyStats = false;
    bool hasAcc = false;
    bool debug = false;
    bool energy = false;
    bool unifiedMem = false;
    bool nodeActivity = false;
    std::string input;
    std::string output;
    std::string energyFile;
    std::string energyStats;
    int sourceNode = 0;
    int deviceID = 0;
    int numberOfItrs = 1;
    float acc = 0.01f;
    Variant variant = ASYNC_PUSH_TD;
    // extensions
    unsigned int partSize = Part_Size;
    float tolerance = 1e-7f;
    unsigned int timeoutMs = 10000;
    unsigned int blocksPerSM = 0;
    unsigned int delta = 0;        // eeg_options.delta
    bool ccComponents = false;     // eeg_options.cc_components
    unsigned long long streamBudgetMiB = 0;  // > 0: eeg_stream_* with this device budget

    ArgumentParser(int argc, char** argv, bool canHaveSource, bool canHaveItrs);
    bool Parse();
    std::string GenerateHelpString();
    // Non-exiting parse used by library callers; returns false with a message instead of exit(0).
    static bool TryParse(int argc, char** argv, bool canHaveSource, bool canHaveItrs, ArgumentParser* out,
                         std::string* error);

   private:
    ArgumentParser() = default;
    bool parse_impl(std::string* error);
};

namespace utilities {
void PrintResults(uint* results, uint n);
void PrintResults(float* results, uint n);
void SaveResults(std::string filepath, uint* results, uint n);
void SaveResults(std::string filepath, float* results, uint n);
void CompareArrays(unsigned int* arr1, unsigned int* arr2, int n);
void CompareArrays(float* arr1, float* arr2, int n);
double maxActivePct(std::vector<unsigned int> activeNodes, unsigned int total);
double pctIterOverThreshold(std::vector<unsigned int> activeNodes, unsigned int total, double threshold);
}  // namespace utilities

// Library entry points (include/eegraph.cuh:21-39). Each builds the virtual graph on the GPU, runs
// the selected variant in one persistent launch, prints the reference's three timing lines, and
// honours --debug / --activity / --output / --energy. Unlike the reference they do not modify
// `graph` (repeated calls on one Graph are safe) and they throw std::runtime_error on CUDA errors
// instead of exiting. PageRank's --output writes the rank values (the reference writes the residual).
Result eegraph_bfs(ArgumentParser& arguments, Graph& graph);
Result eegraph_bfs_um(ArgumentParser& arguments, UMGraph& graph);
Result eegraph_cc(ArgumentParser& arguments, Graph& graph);
Result eegraph_cc_um(ArgumentParser& arguments, UMGraph& graph);
Result eegraph_pr(ArgumentParser& arguments, Graph& graph);
Result eegraph_pr_um(ArgumentParser& arguments, UMGraph& graph);
Result eegraph_sswp(ArgumentParser& arguments, Graph& graph);
Result eegraph_sswp_um(ArgumentParser& arguments, UMGraph& graph);
Result eegraph_sssp(ArgumentParser& arguments, Graph& graph);
Result eegraph_sssp_um(ArgumentParser& arguments, UMGraph& graph);

#endif  // EEGRAPH_HPP
