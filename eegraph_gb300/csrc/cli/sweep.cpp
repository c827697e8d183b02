// sweep.cpp -- sweep-main, the measurement sweep of the reference's src/main.cu:16-493: for every input
// graph, every memory framework (device memory "classic", unified memory "um"), every algorithm, first
// without and then with energy measurement, every trial and every variant, one eegraph_<algo> call whose
// standard output goes to <out>/<algo>/<bench>[-energy]/<variant><trial> (unified-memory runs: variant
// prefixed "um-"), with the energy trace and summary beside it as <variant>-readings<trial> and
// <variant>-stats<trial>. The graphs, their short names, the trial count and the subsets are given on
// the command line instead of the reference's fixed dataset paths; the directory layout and file names
// are the reference's, so its scripts read the results.
#include <filesystem>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "eegraph.hpp"

namespace {

std::vector<std::string> split(const std::string& s) {
    std::vector<std::string> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, ','))
        if (!item.empty()) out.push_back(item);
    return out;
}

const char* kUsage =
    "usage: sweep-main --graphs a.el[,b.el...] [--names a[,b...]] [--trials 5]\n"
    "                  [--frameworks classic,um] [--algos bfs,cc,pr,sssp,sswp] [--energy both|off|on]\n"
    "                  [--variants async-push-td,async-push-dd,sync-push-td,sync-push-dd]\n"
    "                  [--source 0] [--activity] [--out .]\n"
    "Writes <out>/<algo>/<name>[-energy]/<variant><trial> (the program's output of each run; unified-\n"
    "memory runs prefix the variant with um-) and, with energy, <variant>-readings<trial> and\n"
    "<variant>-stats<trial>.\n";

struct VariantName {
    const char* name;
    Variant v;
};
const VariantName kVariants[] = {{"async-push-td", ASYNC_PUSH_TD},
                                 {"async-push-dd", ASYNC_PUSH_DD},
                                 {"sync-push-td", SYNC_PUSH_TD},
                                 {"sync-push-dd", SYNC_PUSH_DD}};

template <class G>
Result run_algo(const std::string& algo, ArgumentParser& args, G& graph);
template <>
Result run_algo<Graph>(const std::string& algo, ArgumentParser& args, Graph& g) {
    if (algo == "bfs") return eegraph_bfs(args, g);
    if (algo == "cc") return eegraph_cc(args, g);
    if (algo == "pr") return eegraph_pr(args, g);
    if (algo == "sssp") return eegraph_sssp(args, g);
    return eegraph_sswp(args, g);
}
template <>
Result run_algo<UMGraph>(const std::string& algo, ArgumentParser& args, UMGraph& g) {
    if (algo == "bfs") return eegraph_bfs_um(args, g);
    if (algo == "cc") return eegraph_cc_um(args, g);
    if (algo == "pr") return eegraph_pr_um(args, g);
    if (algo == "sssp") return eegraph_sssp_um(args, g);
    return eegraph_sswp_um(args, g);
}

struct Plan {
    std::vector<std::string> algos{"bfs", "cc", "pr", "sssp", "sswp"};
    std::vector<std::string> variants{"async-push-td", "async-push-dd", "sync-push-td", "sync-push-dd"};
    std::vector<bool> energy{false, true};
    int trials = 5;
    std::string source = "0";
    bool activity = false;
    std::string out = ".";
};

// One (graph, framework) block of the sweep. Returns the number of runs that raised an error.
template <class G>
int sweep_graph(G& graph, const std::string& input, const std::string& bench, const std::string& prefix,
                const Plan& plan) {
    int failures = 0;
    for (bool energy : plan.energy) {
        for (const std::string& algo : plan.algos) {
            const std::string dir = plan.out + "/" + algo + "/" + bench + (energy ? "-energy" : "") + "/";
            std::filesystem::create_directories(dir);
            for (int trial = 0; trial < plan.trials; ++trial) {
                for (const std::string& vname : plan.variants) {
                    Variant v = ASYNC_PUSH_TD;
                    for (const auto& kv : kVariants)
                        if (vname == kv.name) v = kv.v;
                    // the parser of the per-algorithm programs, with the sweep's settings
                    std::vector<std::string> argv_s{"sweep-main", "--input", input, "--source", plan.source};
                    std::vector<char*> argv;
                    for (auto& a : argv_s) argv.push_back(&a[0]);
                    ArgumentParser args((int)argv.size(), argv.data(), true, false);
                    args.variant = v;
                    args.energy = energy;
                    args.nodeActivity = plan.activity;
                    args.hasEnergyFile = args.hasEnergyStats = energy;
                    const std::string tag = prefix + vname;
                    if (energy) {
                        args.energyFile = dir + tag + "-readings" + std::to_string(trial);
                        args.energyStats = dir + tag + "-stats" + std::to_string(trial);
                    }
                    std::ofstream file(dir + tag + std::to_string(trial));
                    std::streambuf* saved = std::cout.rdbuf(file.rdbuf());
                    try {
                        Result r = run_algo(algo, args, graph);
                        if (plan.activity) {
                            std::cout << "Max active pct: " << utilities::maxActivePct(r.sumLabelsVec, graph.num_nodes)
                                      << std::endl;
                            std::cout << "Pct over threshold: "
                                      << utilities::pctIterOverThreshold(r.sumLabelsVec, graph.num_nodes, .50)
                                      << std::endl;
                        }
                    } catch (const std::exception& e) {
                        std::cout << "error: " << e.what() << std::endl;
                        ++failures;
                    }
                    std::cout.rdbuf(saved);
                }
            }
        }
    }
    return failures;
}

}  // namespace

int main(int argc, char** argv) {
    Plan plan;
    std::vector<std::string> graphs, names;
    std::vector<std::string> frameworks{"classic", "um"};
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&]() -> std::string {
            if (i + 1 >= argc) {
                std::cerr << "missing value after " << a << "\n" << kUsage;
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "--help" || a == "-h") {
            std::cout << kUsage;
            return 0;
        } else if (a == "--graphs") graphs = split(next());
        else if (a == "--names") names = split(next());
        else if (a == "--trials") plan.trials = std::stoi(next());
        else if (a == "--frameworks") frameworks = split(next());
        else if (a == "--algos") plan.algos = split(next());
        else if (a == "--variants") plan.variants = split(next());
        else if (a == "--source") plan.source = next();
        else if (a == "--out") plan.out = next();
        else if (a == "--activity") plan.activity = true;
        else if (a == "--energy") {
            const std::string e = next();
            if (e == "off") plan.energy = {false};
            else if (e == "on") plan.energy = {true};
            else plan.energy = {false, true};
        } else {
            std::cerr << "unknown option " << a << "\n" << kUsage;
            return 2;
        }
    }
    if (graphs.empty()) {
        std::cerr << kUsage;
        return 2;
    }
    for (const auto& v : plan.variants) {
        bool ok = false;
        for (const auto& kv : kVariants) ok = ok || v == kv.name;
        if (!ok) {
            std::cerr << "unknown variant " << v << "\n" << kUsage;
            return 2;
        }
    }
    int failures = 0;
    for (size_t i = 0; i < graphs.size(); ++i) {
        std::string bench = i < names.size() ? names[i] : std::filesystem::path(graphs[i]).stem().string();
        for (const std::string& fw : frameworks) {
            if (fw == "classic") {
                std::cout << "---graph---" << std::endl;
                Graph graph(graphs[i], true);
                graph.ReadGraph();
                failures += sweep_graph(graph, graphs[i], bench, "", plan);
            } else if (fw == "um") {
                std::cout << "---um graph---" << std::endl;
                UMGraph graph(graphs[i], true);
                graph.ReadGraph();
                failures += sweep_graph(graph, graphs[i], bench, "um-", plan);
            } else {
                std::cerr << "unknown framework " << fw << "\n";
                return 2;
            }
        }
    }
    return failures ? 1 : 0;
}
