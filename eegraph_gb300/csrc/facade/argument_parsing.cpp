// argument_parsing.cpp -- ArgumentParser of the C++ facade (reference src/argument_parsing.cpp:1-176).
// Same flags, defaults (source 0, device 0, accuracy 0.01, variant async_push_td) and pair-wise
// parsing (an even argc is an error). Parse() keeps the reference's reaction to a bad command line:
// help text on stdout and exit(0). TryParse() reports the same conditions without exiting.
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "eegraph.hpp"

namespace {
bool is_true(const char* s) { return !strcmp(s, "true") || !strcmp(s, "True") || !strcmp(s, "TRUE"); }
}  // namespace

ArgumentParser::ArgumentParser(int argc_, char** argv_, bool canSource, bool canItrs)
    : argc(argc_), argv(argv_), canHaveSource(canSource), canHaveItrs(canItrs) {
    Parse();
}

bool ArgumentParser::TryParse(int argc_, char** argv_, bool canSource, bool canItrs, ArgumentParser* out,
                              std::string* error) {
    ArgumentParser p;
    p.argc = argc_;
    p.argv = argv_;
    p.canHaveSource = canSource;
    p.canHaveItrs = canItrs;
    std::string err;
    const bool ok = p.parse_impl(&err);
    if (error) *error = err;
    if (ok && out) *out = p;
    return ok;
}

bool ArgumentParser::Parse() {
    std::string err;
    if (!parse_impl(&err)) {
        std::cout << err;
        exit(0);
    }
    return true;
}

bool ArgumentParser::parse_impl(std::string* error) {
    if (argc == 1) {
        *error = GenerateHelpString();
        return false;
    }
    if (argc == 2 && (!strcmp(argv[1], "--help") || !strcmp(argv[1], "-help") || !strcmp(argv[1], "--h") ||
                      !strcmp(argv[1], "-h"))) {
        *error = GenerateHelpString();
        return false;
    }
    if (argc % 2 == 0) {
        *error = "\nThere was an error parsing command line arguments\n" + GenerateHelpString();
        return false;
    }
    for (int i = 1; i < argc - 1; i += 2) {
        const char* k = argv[i];
        const char* v = argv[i + 1];
        if (!strcmp(k, "--input")) {
            input = v;
            hasInput = true;
        } else if (!strcmp(k, "--output")) {
            output = v;
            hasOutput = true;
        } else if (!strcmp(k, "--efile")) {
            energyFile = v;
            hasEnergyFile = true;
        } else if (!strcmp(k, "--estats")) {
            energyStats = v;
            hasEnergyStats = true;
        } else if (!strcmp(k, "--source") && canHaveSource) {
            sourceNode = atoi(v);
            hasSourceNode = true;
        } else if (!strcmp(k, "--device")) {
            deviceID = atoi(v);
            hasDeviceID = true;
        } else if (!strcmp(k, "--iteration") && canHaveItrs) {
            numberOfItrs = atoi(v);
            hasNumberOfItrs = true;
        } else if (!strcmp(k, "--debug")) {
            if (is_true(v)) debug = true;
        } else if (!strcmp(k, "--activity")) {
            if (is_true(v)) nodeActivity = true;
        } else if (!strcmp(k, "--variant")) {
            if (!strcmp(v, "async_push_td")) variant = ASYNC_PUSH_TD;
            else if (!strcmp(v, "async_push_dd")) variant = ASYNC_PUSH_DD;
            else if (!strcmp(v, "sync_push_td")) variant = SYNC_PUSH_TD;
            else if (!strcmp(v, "sync_push_dd")) variant = SYNC_PUSH_DD;
            else {
                *error = "Variant not recognized\n";
                return false;
            }
        } else if (!strcmp(k, "--energy")) {
            if (is_true(v)) energy = true;
        } else if (!strcmp(k, "--um")) {
            if (is_true(v)) unifiedMem = true;
        } else if (!strcmp(k, "--accuracy")) {
            acc = (float)atof(v);
            hasAcc = true;
        } else if (!strcmp(k, "--k")) {
            partSize = (unsigned)atoi(v);
            if (partSize != 4 && partSize != 8 && partSize != 16) {
                *error = "--k must be 4, 8 or 16\n";
                return false;
            }
        } else if (!strcmp(k, "--tolerance")) {
            tolerance = (float)atof(v);
        } else if (!strcmp(k, "--timeout")) {
            timeoutMs = (unsigned)atoi(v);
        } else if (!strcmp(k, "--blocks-per-sm")) {
            blocksPerSM = (unsigned)atoi(v);
        } else if (!strcmp(k, "--delta")) {
            delta = (unsigned)atoi(v);
        } else if (!strcmp(k, "--cc-components")) {
            ccComponents = is_true(v);
        } else if (!strcmp(k, "--stream-budget")) {
            streamBudgetMiB = strtoull(v, nullptr, 10);
        } else {
            *error = std::string("\nThere was an error parsing command line argument <") + k + ">\n" +
                     GenerateHelpString();
            return false;
        }
    }
    if (energy && (!hasEnergyFile || !hasEnergyStats)) {
        *error = "The option --energy was true but energy file and/or energy stats files were not included\n";
        return false;
    }
    if (!hasInput) {
        *error = "\nInput graph file argument is required.\n" + GenerateHelpString();
        return false;
    }
    return true;
}

std::string ArgumentParser::GenerateHelpString() {
    std::string str = "\nRequired arguments:";
    str += "\n    [--input]: Input graph file. E.g., --input FacebookGraph.txt";
    str += "\nOptional arguments";
    if (canHaveSource) str += "\n    [--source]:  Begins from the source (Default: 0). E.g., --source 10";
    str += "\n    [--output]: Output file for results. E.g., --output results.txt";
    str += "\n    [--device]: Select GPU device (Default: 0). E.g., --device 1";
    if (canHaveItrs) str += "\n    [--iteration]: Number of iterations (Default: 1). E.g., --iteration 10";
    str += "\n    [--debug]: Check or observe information (Default: false). E.g. --debug true";
    str += "\n    [--variant]: Algorithm variant option (Default: async_push_td). E.g. --variant async_push_td";
    str += "\n    [--energy]: Measure and output GPU energy information (Default: false). E.g. --energy true";
    str += "\n    [--efile]: Output file for energy (Required if energy == true). E.g. --efile my_experiment_energy";
    str += "\n    [--estats]: Output file for energy (Required if energy == true). E.g. --estats my_experiment_stats";
    str += "\n    [--um]: Use unified memory for graph algorithms. E.g. --um true";
    str += "\n    [--accuracy]: PageRank activation threshold. E.g. --accuracy 0.01";
    str += "\n    [--activity]: sum node activity vector in results (Default false) E.g. --activity true";
    str += "\n    [--k]: virtual-node size K, 4, 8 or 16 (Default: 8). E.g. --k 16";
    str += "\n    [--tolerance]: PageRank bound on ||x - x*||_1 / ||x||_1 (Default: 1e-7)";
    str += "\n    [--timeout]: bound on any device-side wait in ms (Default: 10000)";
    str += "\n    [--blocks-per-sm]: cap on resident CTAs per SM for the persistent kernels";
    str += "\n    [--delta]: SSSP/SSWP sync-push-dd bucketed rounds of this key width (Default: 0 = plain)";
    str += "\n    [--cc-components]: CC as connected components, relaxing with weight 0 (Default: false)";
    str += "\n    [--stream-budget]: MiB of device buffers; > 0 keeps the graph in host memory and streams each "
           "round's active subgraph (BFS/SSSP/SSWP/CC; Default: 0 = graph on the device)";
    str += "\n\n";
    return str;
}
