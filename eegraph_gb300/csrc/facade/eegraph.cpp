// eegraph.cpp -- eegraph_<algo>[_um] entry points of the C++ facade (reference src/eegraph.cu:1-2540,
// declared in include/eegraph.cuh:21-39).
//
// Each call: optional energy session (NVML), device selection (--device), GPU build of the virtual
// graph (lossless), one persistent launch of the chosen variant, copy-back of the result, the
// reference's console lines, then --debug (sequential host check, first 30 values, first mismatch),
// --activity (per-iteration active-vertex counts) and --output ("i value" lines).
#include <algorithm>
#include <deque>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "eegraph.hpp"

namespace {

void check(eeg_status s, const char* what) {
    if (s != EEG_OK) throw std::runtime_error(std::string(what) + ": " + eeg_status_string(s) + " -- " + eeg_last_error());
}

// Sequential label-correcting check used by --debug (the reference recomputes with seq_cpu on the
// host, src/eegraph.cu:239-257). BFS/SSSP/CC: min-plus; SSWP: max-min. seed_all selects the initial
// active set (every vertex, or the source only).
std::vector<uint> host_check(eeg_algo algo, bool seed_all, uint n, const std::vector<uint32_t>& s,
                             const std::vector<uint32_t>& d, const std::vector<uint32_t>& w, uint source) {
    std::vector<uint> val(n);
    for (uint v = 0; v < n; ++v) {
        if (algo == EEG_CC) val[v] = v;
        else if (algo == EEG_SSWP) val[v] = v == source ? DIST_INFINITY : 0u;
        else val[v] = v == source ? 0u : DIST_INFINITY;
    }
    std::vector<uint64_t> off(n + 1, 0);
    for (size_t e = 0; e < s.size(); ++e) off[s[e] + 1]++;
    for (uint v = 0; v < n; ++v) off[v + 1] += off[v];
    std::vector<uint32_t> col(s.size()), wt(s.size());
    std::vector<uint64_t> pos(off.begin(), off.end() - 1);
    for (size_t e = 0; e < s.size(); ++e) {
        col[pos[s[e]]] = d[e];
        wt[pos[s[e]]++] = w.empty() ? 1u : w[e];
    }
    std::deque<uint> work;
    std::vector<char> inq(n, 0);
    if (seed_all) {
        for (uint v = 0; v < n; ++v) work.push_back(v), inq[v] = 1;
    } else {
        work.push_back(source);
        inq[source] = 1;
    }
    while (!work.empty()) {
        const uint u = work.front();
        work.pop_front();
        inq[u] = 0;
        const uint du = val[u];
        if ((algo == EEG_BFS || algo == EEG_SSSP) && du == DIST_INFINITY) continue;
        if (algo == EEG_SSWP && du == 0) continue;
        for (uint64_t e = off[u]; e < off[u + 1]; ++e) {
            const uint t = col[e];
            uint nd;
            bool better;
            if (algo == EEG_SSWP) {
                nd = std::min(du, wt[e]);
                better = nd > val[t];
            } else {
                const uint64_t x = (uint64_t)du + (algo == EEG_BFS ? 1u : wt[e]);
                nd = x >= DIST_INFINITY ? DIST_INFINITY : (uint)x;
                better = nd < val[t];
            }
            if (better) {
                val[t] = nd;
                if (!inq[t]) work.push_back(t), inq[t] = 1;
            }
        }
    }
    return val;
}

struct EdgeArrays {
    std::vector<uint32_t> s, d, w;
};

template <class G>
EdgeArrays normalized_edges(const G& g) {
    // 1-based files: ids shifted down by one (src/virtual_graph.cpp:5-12), without touching `g`
    const uint32_t shift = g.hasZeroID ? 0u : 1u;
    EdgeArrays a;
    a.s.resize(g.num_edges);
    a.d.resize(g.num_edges);
    a.w.resize(g.num_edges);
    for (uint e = 0; e < g.num_edges; ++e) {
        a.s[e] = g.edges[e].source - shift;
        a.d[e] = g.edges[e].end - shift;
    }
    return a;
}

template <class G>
const uint* weights_of(const G& g);
template <>
const uint* weights_of<Graph>(const Graph& g) {
    return g.weights.size() == g.edges.size() && !g.weights.empty() ? g.weights.data() : nullptr;
}
template <>
const uint* weights_of<UMGraph>(const UMGraph& g) {
    return g.weights;
}

template <class G>
Result run_algo(ArgumentParser& args, G& graph, eeg_algo algo, bool um) {
    if (um) std::cout << "Unified memory version" << std::endl;
    eeg_energy* en = nullptr;
    if (args.energy) {
        std::cout << "Starting energy measurements. Timing information will be affected..." << std::endl;
        if (eeg_energy_begin(args.deviceID, args.energyFile.c_str(), 1000, &en) != EEG_OK) {
            std::cout << "Energy unavailable: " << eeg_last_error() << std::endl;
            en = nullptr;
        }
    }
    if (args.hasDeviceID) check(eeg_set_device(args.deviceID), "cudaSetDevice");
    const uint n = graph.num_nodes;
    if (n == 0) throw std::invalid_argument("graph has no vertices (was ReadGraph called?)");
    if (algo != EEG_PR && (args.sourceNode < 0 || (uint)args.sourceNode >= n))
        throw std::invalid_argument("source vertex out of range");
    EdgeArrays ea = normalized_edges(graph);
    const uint* w = weights_of(graph);
    for (uint e = 0; e < graph.num_edges; ++e) ea.w[e] = w ? w[e] : 1u;

    Timer totalTimer;
    totalTimer.Start();
    if (en) eeg_energy_mark(en);
    // --stream-budget: the graph stays in host memory and each round's active subgraph is streamed
    eeg_stream* sg = nullptr;
    if (args.streamBudgetMiB > 0) {
        if (algo == EEG_PR) throw std::invalid_argument("--stream-budget: PageRank is not streamed");
        eeg_graph* hg = nullptr;
        check(eeg_graph_from_arrays(n, graph.num_edges, ea.s.data(), ea.d.data(), ea.w.data(), &hg), "host graph");
        const eeg_status cs = eeg_stream_create(hg, args.partSize, args.streamBudgetMiB << 20, &sg);
        eeg_graph_destroy(hg);
        check(cs, "streamed graph");
    }
    // PageRank's topology-driven pull reads only the transposed graph and the out-degrees; its data-driven
    // variants push along out-edges, so they get the forward parts as well
    const bool pr_dd = algo == EEG_PR && (args.variant == SYNC_PUSH_DD || args.variant == ASYNC_PUSH_DD);
    uint32_t flags = (algo == EEG_PR ? (uint32_t)(pr_dd ? EEG_VG_REVERSE : EEG_VG_REVERSE_ONLY) : 0u) |
                     (um ? (uint32_t)EEG_VG_MANAGED : 0u);
    eeg_vgraph* vg = nullptr;
    if (!sg)
        check(eeg_vgraph_build_arrays(n, graph.num_edges, ea.s.data(), ea.d.data(), ea.w.data(), args.partSize, flags,
                                      nullptr, &vg),
              "virtual graph build");

    eeg_options o;
    eeg_options_init(&o);
    o.pr_tolerance = args.tolerance;
    o.pr_accuracy = args.hasAcc ? args.acc : 0.f;
    o.timeout_ms = args.timeoutMs;
    o.blocks_per_sm = args.blocksPerSM;
    o.delta = args.delta;
    o.cc_components = args.ccComponents ? 1u : 0u;
    Result result;
    std::vector<uint> dist;
    std::vector<float> rank;
    if (algo == EEG_PR) rank.resize(n);
    else dist.resize(n);
    std::vector<uint32_t> activity(args.nodeActivity ? std::max<uint>(n + 2, 1024) : 0);
    eeg_result r;
    Timer timer;
    timer.Start();
    if (en) eeg_energy_mark(en);
    eeg_status s;
    if (sg) {
        s = eeg_stream_run(sg, algo, (eeg_variant)args.variant, (uint32_t)args.sourceNode, &o, dist.data(), 0, nullptr,
                           &r);
    } else {
        s = eeg_run(vg, algo, (eeg_variant)args.variant, (uint32_t)args.sourceNode, &o,
                    algo == EEG_PR ? (void*)rank.data() : (void*)dist.data(), 0,
                    args.nodeActivity ? activity.data() : nullptr, (uint32_t)activity.size(), nullptr, &r);
    }
    if (en) eeg_energy_mark(en);
    const float runtime = timer.Finish();
    const float total = totalTimer.Finish();
    if (vg) eeg_vgraph_destroy(vg);
    if (sg) eeg_stream_destroy(sg);
    if (s != EEG_OK) {
        if (en) eeg_energy_destroy(en);
        check(s, "run");
    }
    std::cout << "Number of iterations = " << r.iterations << std::endl;
    std::cout << "Processing finished in " << runtime << " (ms).\n";
    std::cout << "Total GPU activity finished in " << total << " (ms).\n";

    result.time = total;
    result.processingTime = r.kernel_ms;
    result.iterations = r.iterations;
    result.gteps = r.gteps;
    result.algorithmicBytes = r.algorithmic_bytes;
    result.reachedVertices = r.reached_vertices;
    result.reachedEdges = r.reached_edges;
    result.energy = -1.0;
    if (en) {
        double j = 0, sec = 0, watts = 0;
        if (eeg_energy_end(en, &j, &sec, &watts) == EEG_OK) {
            result.energy = j;
            std::cout << "Energy consumed = " << j << " (J) over " << sec << " (s), average " << watts << " (W)\n";
            if (args.hasEnergyStats) {
                std::ofstream st(args.energyStats);
                st << "energy_j,seconds,avg_w,processing_ms,total_ms\n" << j << "," << sec << "," << watts << ","
                   << runtime << "," << total << "\n";
            }
        } else {
            std::cout << "Energy unavailable: " << eeg_last_error() << std::endl;
        }
        eeg_energy_destroy(en);
    }
    if (args.nodeActivity) result.sumLabelsVec.assign(activity.begin(), activity.begin() + r.num_activity);

    if (args.debug) {
        if (algo == EEG_PR) {
            utilities::PrintResults(rank.data(), std::min<uint>(30, n));
        } else {
            // CC seeds every vertex, except SYNC_PUSH_DD on the device graph (src/eegraph.cu:548-553)
            const bool seed_all = args.streamBudgetMiB > 0 || !(args.variant == SYNC_PUSH_DD) || algo != EEG_CC;
            std::vector<uint> cpu = host_check(algo, algo == EEG_CC ? seed_all : false, n, ea.s, ea.d, ea.w,
                                               (uint)args.sourceNode);
            utilities::PrintResults(cpu.data(), std::min<uint>(30, n));
            utilities::PrintResults(dist.data(), std::min<uint>(30, n));
            utilities::CompareArrays(cpu.data(), dist.data(), (int)n);
        }
    }
    if (args.hasOutput) {
        if (algo == EEG_PR) utilities::SaveResults(args.output, rank.data(), n);
        else utilities::SaveResults(args.output, dist.data(), n);
    }
    return result;
}

}  // namespace

Result eegraph_bfs(ArgumentParser& a, Graph& g) { return run_algo(a, g, EEG_BFS, false); }
Result eegraph_bfs_um(ArgumentParser& a, UMGraph& g) { return run_algo(a, g, EEG_BFS, true); }
Result eegraph_cc(ArgumentParser& a, Graph& g) { return run_algo(a, g, EEG_CC, false); }
Result eegraph_cc_um(ArgumentParser& a, UMGraph& g) { return run_algo(a, g, EEG_CC, true); }
Result eegraph_pr(ArgumentParser& a, Graph& g) { return run_algo(a, g, EEG_PR, false); }
Result eegraph_pr_um(ArgumentParser& a, UMGraph& g) { return run_algo(a, g, EEG_PR, true); }
Result eegraph_sswp(ArgumentParser& a, Graph& g) { return run_algo(a, g, EEG_SSWP, false); }
Result eegraph_sswp_um(ArgumentParser& a, UMGraph& g) { return run_algo(a, g, EEG_SSWP, true); }
Result eegraph_sssp(ArgumentParser& a, Graph& g) { return run_algo(a, g, EEG_SSSP, false); }
Result eegraph_sssp_um(ArgumentParser& a, UMGraph& g) { return run_algo(a, g, EEG_SSSP, true); }
