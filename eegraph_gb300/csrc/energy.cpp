// energy.cpp -- GPU energy of a region through NVML, loaded at run time.
//
// Replaces nvmlClass (reference include/nvmlClass.cuh:77-356): that class polls power every 50 us on a
// thread and integrates it between markers, with 5 s of warm-up and cool-down sampling around the
// run. Here the primary source is NVML's total-energy counter (millijoules since driver load), read
// at begin and end, so a run costs two NVML calls and no polling thread perturbs the timing. A
// power-sampling thread runs only when a CSV trace is requested, or when the counter is not
// supported (then the samples are integrated with the trapezoid rule). Without libnvidia-ml the
// calls return EEG_ERR_ENERGY and callers report "energy unavailable" instead of aborting.
#include <dlfcn.h>
#include <nvml.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "internal.hpp"

namespace {

struct NvmlApi {
    void* lib = nullptr;
    nvmlReturn_t (*init)() = nullptr;
    nvmlReturn_t (*shutdown)() = nullptr;
    nvmlReturn_t (*by_pci)(const char*, nvmlDevice_t*) = nullptr;
    nvmlReturn_t (*by_index)(unsigned int, nvmlDevice_t*) = nullptr;
    nvmlReturn_t (*energy)(nvmlDevice_t, unsigned long long*) = nullptr;
    nvmlReturn_t (*power)(nvmlDevice_t, unsigned int*) = nullptr;
    bool ok = false;
};

std::mutex g_mu;
NvmlApi g_api;
int g_refs = 0;

bool nvml_acquire(std::string& why) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_refs > 0) {
        ++g_refs;
        return true;
    }
    if (!g_api.lib) {
        const char* env = getenv("EEG_NVML_LIBRARY");  // tests point this at a fake NVML
        g_api.lib = dlopen(env && *env ? env : "libnvidia-ml.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!g_api.lib) {
            why = "libnvidia-ml.so.1 not found";
            return false;
        }
        g_api.init = (nvmlReturn_t(*)())dlsym(g_api.lib, "nvmlInit_v2");
        g_api.shutdown = (nvmlReturn_t(*)())dlsym(g_api.lib, "nvmlShutdown");
        g_api.by_pci = (nvmlReturn_t(*)(const char*, nvmlDevice_t*))dlsym(g_api.lib, "nvmlDeviceGetHandleByPciBusId_v2");
        g_api.by_index = (nvmlReturn_t(*)(unsigned int, nvmlDevice_t*))dlsym(g_api.lib, "nvmlDeviceGetHandleByIndex_v2");
        g_api.energy = (nvmlReturn_t(*)(nvmlDevice_t, unsigned long long*))dlsym(g_api.lib, "nvmlDeviceGetTotalEnergyConsumption");
        g_api.power = (nvmlReturn_t(*)(nvmlDevice_t, unsigned int*))dlsym(g_api.lib, "nvmlDeviceGetPowerUsage");
        g_api.ok = g_api.init && g_api.shutdown && (g_api.by_pci || g_api.by_index) && (g_api.energy || g_api.power);
    }
    if (!g_api.ok) {
        why = "NVML library lacks required symbols";
        return false;
    }
    if (g_api.init() != NVML_SUCCESS) {
        why = "nvmlInit failed";
        return false;
    }
    g_refs = 1;
    return true;
}

void nvml_release() {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_refs > 0 && --g_refs == 0) g_api.shutdown();
}

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct eeg_energy {
    nvmlDevice_t dev{};
    bool have_counter = false;
    unsigned long long e0 = 0;
    double t0 = 0.0;
    std::vector<std::pair<double, double>> samples;  // (s, W)
    std::vector<double> marks;
    std::mutex mu;
    std::atomic<bool> stop{false};
    std::thread sampler;
    FILE* csv = nullptr;
    uint32_t period_us = 1000;
};

extern "C" {

EEG_API eeg_status eeg_energy_begin(int device, const char* csv_path, uint32_t sample_period_us, eeg_energy** out) {
    if (!out) {
        eeg::set_last_error("null output handle");
        return EEG_ERR_INVALID;
    }
    *out = nullptr;
    std::string why;
    if (!nvml_acquire(why)) {
        eeg::set_last_error("energy unavailable: " + why);
        return EEG_ERR_ENERGY;
    }
    eeg_energy* e = new eeg_energy();
    bool have_dev = false;
    char bus[32] = {0};
    if (g_api.by_pci && cudaDeviceGetPCIBusId(bus, sizeof(bus), device) == cudaSuccess)
        have_dev = g_api.by_pci(bus, &e->dev) == NVML_SUCCESS;
    (void)cudaGetLastError();
    if (!have_dev && g_api.by_index) have_dev = g_api.by_index((unsigned)device, &e->dev) == NVML_SUCCESS;
    if (!have_dev) {
        delete e;
        nvml_release();
        eeg::set_last_error("energy unavailable: NVML has no handle for the device");
        return EEG_ERR_ENERGY;
    }
    e->period_us = sample_period_us ? sample_period_us : 1000u;
    e->have_counter = g_api.energy && g_api.energy(e->dev, &e->e0) == NVML_SUCCESS;
    e->t0 = now_s();
    if (csv_path && *csv_path) {
        e->csv = fopen(csv_path, "w");
        if (e->csv) fprintf(e->csv, "time_s,power_w\n");
    }
    if ((e->csv || !e->have_counter) && g_api.power) {
        e->sampler = std::thread([e] {
            while (!e->stop.load()) {
                unsigned int mw = 0;
                if (g_api.power(e->dev, &mw) == NVML_SUCCESS) {
                    const double t = now_s() - e->t0;
                    std::lock_guard<std::mutex> lk(e->mu);
                    e->samples.emplace_back(t, mw / 1000.0);
                    if (e->csv) fprintf(e->csv, "%.6f,%.3f\n", t, mw / 1000.0);
                }
                std::this_thread::sleep_for(std::chrono::microseconds(e->period_us));
            }
        });
    } else if (!e->have_counter) {
        delete e;
        nvml_release();
        eeg::set_last_error("energy unavailable: neither the energy counter nor power readings work");
        return EEG_ERR_ENERGY;
    }
    *out = e;
    return EEG_OK;
}

EEG_API eeg_status eeg_energy_mark(eeg_energy* e) {
    if (!e) {
        eeg::set_last_error("null handle");
        return EEG_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(e->mu);
    const double t = now_s() - e->t0;
    e->marks.push_back(t);
    if (e->csv) fprintf(e->csv, "# mark %.6f\n", t);
    return EEG_OK;
}

EEG_API eeg_status eeg_energy_end(eeg_energy* e, double* joules, double* seconds, double* avg_watts) {
    if (!e) {
        eeg::set_last_error("null handle");
        return EEG_ERR_INVALID;
    }
    unsigned long long e1 = 0;
    const bool counter = e->have_counter && g_api.energy(e->dev, &e1) == NVML_SUCCESS;
    const double dt = now_s() - e->t0;
    if (e->sampler.joinable()) {
        e->stop.store(true);
        e->sampler.join();
    }
    double j = 0.0;
    if (counter) {
        j = (double)(e1 - e->e0) / 1000.0;
    } else {
        std::lock_guard<std::mutex> lk(e->mu);
        for (size_t i = 1; i < e->samples.size(); ++i)
            j += 0.5 * (e->samples[i].second + e->samples[i - 1].second) * (e->samples[i].first - e->samples[i - 1].first);
        if (e->samples.size() < 2) {
            eeg::set_last_error("energy unavailable: too few power samples");
            return EEG_ERR_ENERGY;
        }
    }
    if (joules) *joules = j;
    if (seconds) *seconds = dt;
    if (avg_watts) *avg_watts = dt > 0 ? j / dt : 0.0;
    return EEG_OK;
}

EEG_API void eeg_energy_destroy(eeg_energy* e) {
    if (!e) return;
    if (e->sampler.joinable()) {
        e->stop.store(true);
        e->sampler.join();
    }
    if (e->csv) fclose(e->csv);
    delete e;
    nvml_release();
}

}  // extern "C"
