// converter.cpp -- `converter <file.el|file.wel>`, the text-to-binary CSR converter of Subway
// (Subway/tools/converter.cpp:21-172): X.el becomes X.bcsr and X.wel becomes X.bwcsr beside it.
// The file holds num_nodes = largest id + 1 (ids kept as read: no 1-based shift), num_edges, one
// u32 offset per vertex and the edges grouped by source, in input order within a source. Any other
// extension prints the reference's message, and so does a wrong argument count; both exit 0, as the
// reference does. Unlike the reference, a line that does not start with a digit is skipped (the
// loader's rule, src/graph.cpp:64-105) instead of being read as an edge.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>

#include "eegraph_c.h"

int main(int argc, char** argv) {
    if (argc != 2) {
        std::printf("\nThere was an error parsing command line arguments\n");
        return 0;
    }
    const std::string input = argv[1];
    const size_t dot = input.find_last_of('.');
    const std::string ext = dot == std::string::npos ? "" : input.substr(dot + 1);
    if (ext != "el" && ext != "wel") {
        std::printf("\nInput file format is not supported.\n");
        return 0;
    }
    const bool weighted = ext == "wel";
    eeg_graph* g = nullptr;
    if (eeg_graph_load(input.c_str(), weighted ? 1 : 0, 0, &g) != EEG_OK) {
        std::fprintf(stderr, "converter: %s\n", eeg_last_error());
        return 1;
    }
    eeg_graph_view v{};
    eeg_graph_view_get(g, &v);
    uint32_t largest = 0;
    for (uint64_t e = 0; e < v.num_edges; ++e) largest = std::max(largest, std::max(v.src[e], v.dst[e]));
    if (largest == UINT32_MAX) {
        std::fprintf(stderr, "converter: vertex id 4294967295 does not fit the 32-bit vertex count\n");
        eeg_graph_destroy(g);
        return 1;
    }
    // the ids as read, taken as 0-based, over largest + 1 vertices
    eeg_graph* raw = nullptr;
    eeg_status st = eeg_graph_from_arrays(largest + 1u, v.num_edges, v.src, v.dst, weighted ? v.weight : nullptr, &raw);
    const std::string out = input.substr(0, dot + 1) + (weighted ? "bwcsr" : "bcsr");
    if (st == EEG_OK) st = eeg_graph_save_bcsr(raw, out.c_str());
    if (st != EEG_OK) std::fprintf(stderr, "converter: %s\n", eeg_last_error());
    eeg_graph_destroy(raw);
    eeg_graph_destroy(g);
    return st == EEG_OK ? 0 : 1;
}
