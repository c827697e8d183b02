// utilities.cpp -- result printing/saving helpers of the C++ facade (reference src/utilities.cpp:1-80).
// Output formats are the reference's: "Results of first n nodes:\n[0:v0 1:v1 ...]" and a result
// file of "i value" lines.
#include <fstream>
#include <iostream>

#include "eegraph.hpp"

namespace utilities {

template <class T>
static void print_results(T* results, uint n) {
    std::cout << "Results of first " << n << " nodes:\n[";
    for (uint i = 0; i < n; i++) {
        if (i > 0) std::cout << " ";
        std::cout << i << ":" << results[i];
    }
    std::cout << "]\n";
}

void PrintResults(uint* results, uint n) { print_results(results, n); }
void PrintResults(float* results, uint n) { print_results(results, n); }

void SaveResults(std::string filepath, uint* results, uint n) {
    std::cout << "Saving the results into the following file:\n";
    std::cout << ">> " << filepath << std::endl;
    std::ofstream outfile(filepath);
    for (uint i = 0; i < n; i++) outfile << i << " " << results[i] << "\n";
    std::cout << "Done saving.\n";
}

void SaveResults(std::string filepath, float* results, uint n) {
    std::cout << "Saving the results into " << filepath << " ...... " << std::flush;
    std::ofstream outfile(filepath);
    for (uint i = 0; i < n; i++) outfile << i << " " << results[i] << "\n";
    std::cout << " Completed.\n";
}

template <class T>
static void compare(T* a, T* b, int n) {
    for (int i = 0; i < n; i++) {
        if (a[i] != b[i]) {
            std::cout << "Arrays begin to differ at element " << i << std::endl;
            std::cout << "Arr1[" << i << "]: " << a[i] << std::endl;
            std::cout << "Arr2[" << i << "]: " << b[i] << std::endl;
            break;
        }
    }
}

void CompareArrays(unsigned int* a, unsigned int* b, int n) { compare(a, b, n); }
void CompareArrays(float* a, float* b, int n) { compare(a, b, n); }

double maxActivePct(std::vector<unsigned int> activeNodes, unsigned int total) {
    unsigned int mx = 0;
    for (unsigned int a : activeNodes) mx = a > mx ? a : mx;
    return total ? (double)mx / (double)total : 0.0;
}

double pctIterOverThreshold(std::vector<unsigned int> activeNodes, unsigned int total, double threshold) {
    if (activeNodes.empty() || total == 0) return 0.0;
    unsigned int count = 0;
    for (unsigned int a : activeNodes)
        if ((double)a / (double)total > threshold) count++;
    return (double)count / (double)activeNodes.size();
}

}  // namespace utilities
