// power.cpp -- board power sampling during a run (the reference's
// power_measurer, util_device.cu:78-130): a background thread reads the GPU's
// power draw every `period` ms until stopped and reports the mean in watts.
//
// NVML is loaded at run time (libnvidia-ml.so.1, or the library named by
// GU_NVML_LIBRARY -- tests point it at a fake), through the handful of entry
// points declared here, so nothing needs NVIDIA's header.  The sampler only
// reads: it changes no GPU setting.  The CUDA device is matched to its NVML
// handle by PCI bus id (CUDA_VISIBLE_DEVICES may renumber devices), falling
// back to the same index when the bus id is unavailable.
#include "gu_internal.h"

#include <dlfcn.h>

#include <atomic>
#include <chrono>
#include <cstdlib>
#include <memory>
#include <string>
#include <thread>

namespace gu {

namespace {

typedef int nvml_ret;  // nvmlReturn_t: 0 = success
typedef struct nvml_device_st *nvml_device;

struct Nvml {
    void *so = nullptr;
    nvml_ret (*init)() = nullptr;
    nvml_ret (*shutdown)() = nullptr;
    nvml_ret (*by_index)(unsigned, nvml_device *) = nullptr;
    nvml_ret (*by_pci)(const char *, nvml_device *) = nullptr;
    nvml_ret (*power)(nvml_device, unsigned *) = nullptr;  // milliwatts

    void load()
    {
        const char *name = std::getenv("GU_NVML_LIBRARY");
        so = dlopen(name && *name ? name : "libnvidia-ml.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!so) throw gu_error(GU_ERR_UNSUPPORTED, std::string("NVML is not available: ") + dlerror());
        auto sym = [&](const char *a, const char *b) {
            void *p = dlsym(so, a);
            if (!p && b) p = dlsym(so, b);
            return p;
        };
        init = reinterpret_cast<nvml_ret (*)()>(sym("nvmlInit_v2", "nvmlInit"));
        shutdown = reinterpret_cast<nvml_ret (*)()>(sym("nvmlShutdown", nullptr));
        by_index = reinterpret_cast<nvml_ret (*)(unsigned, nvml_device *)>(
            sym("nvmlDeviceGetHandleByIndex_v2", "nvmlDeviceGetHandleByIndex"));
        by_pci = reinterpret_cast<nvml_ret (*)(const char *, nvml_device *)>(
            sym("nvmlDeviceGetHandleByPciBusId_v2", "nvmlDeviceGetHandleByPciBusId"));
        power = reinterpret_cast<nvml_ret (*)(nvml_device, unsigned *)>(sym("nvmlDeviceGetPowerUsage", nullptr));
        if (!init || !shutdown || !by_index || !power) {
            dlclose(so);
            so = nullptr;
            throw gu_error(GU_ERR_UNSUPPORTED, "NVML library lacks the power entry points");
        }
    }
};

}  // namespace

struct PowerSampler {
    Nvml nv;
    nvml_device dev = nullptr;
    std::atomic<bool> run{true};
    std::thread th;
    double sum_w = 0.0;
    long long samples = 0;
    int period_ms = 10;
    nvml_ret err = 0;

    ~PowerSampler()
    {
        if (th.joinable()) {
            run = false;
            th.join();
        }
        if (nv.so) {
            nv.shutdown();
            dlclose(nv.so);
        }
    }
};

PowerSampler *power_start(int device, int period_ms)
{
    if (period_ms < 1) throw gu_error(GU_ERR_INVALID_ARGUMENT, "period must be >= 1 ms");
    std::unique_ptr<PowerSampler> p(new PowerSampler());
    p->nv.load();
    if (p->nv.init() != 0) throw gu_error(GU_ERR_UNSUPPORTED, "nvmlInit failed");
    char bus[64] = {0};
    bool found = false;
    if (p->nv.by_pci && cudaDeviceGetPCIBusId(bus, sizeof(bus), device) == cudaSuccess)
        found = p->nv.by_pci(bus, &p->dev) == 0;
    cudaGetLastError();  // no CUDA device here is not an error for the fallback
    if (!found && p->nv.by_index((unsigned)device, &p->dev) != 0)
        throw gu_error(GU_ERR_INVALID_ARGUMENT, "no NVML device for CUDA device " + std::to_string(device));
    p->period_ms = period_ms;
    PowerSampler *s = p.get();
    s->th = std::thread([s] {
        while (true) {
            unsigned mw = 0;
            const nvml_ret r = s->nv.power(s->dev, &mw);
            if (r != 0) {
                s->err = r;
                return;
            }
            s->sum_w += mw / 1000.0;
            ++s->samples;
            if (!s->run) return;  // at least one sample, and one after the stop request
            std::this_thread::sleep_for(std::chrono::milliseconds(s->period_ms));
        }
    });
    return p.release();
}

void power_stop(PowerSampler *s, double *avg_w, long long *samples)
{
    s->run = false;
    if (s->th.joinable()) s->th.join();
    const nvml_ret e = s->err;
    const double avg = s->samples ? s->sum_w / (double)s->samples : 0.0;
    const long long n = s->samples;
    delete s;
    if (e != 0) throw gu_error(GU_ERR_UNSUPPORTED, "nvmlDeviceGetPowerUsage failed with code " + std::to_string(e));
    if (avg_w) *avg_w = avg;
    if (samples) *samples = n;
}

}  // namespace gu
