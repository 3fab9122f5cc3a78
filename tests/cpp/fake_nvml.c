/* fake_nvml.c -- a stand-in for the NVML library with the entry points the
 * power sampler uses, for host-only tests: one device, a constant 123.456 W
 * draw, or failing power reads when FAKE_NVML_FAIL is set.  Test infrastructure. */
#include <stdlib.h>

typedef struct fake_device { int id; } fake_device;
static fake_device dev0 = {0};
static int inits = 0;

int nvmlInit_v2(void) { ++inits; return 0; }
int nvmlShutdown(void) { return inits-- > 0 ? 0 : 1; }
int nvmlDeviceGetHandleByIndex_v2(unsigned index, fake_device **d)
{
    if (index != 0) return 2; /* invalid argument */
    *d = &dev0;
    return 0;
}
int nvmlDeviceGetHandleByPciBusId_v2(const char *bus, fake_device **d)
{
    (void)bus;
    *d = &dev0;
    return 0;
}
int nvmlDeviceGetPowerUsage(fake_device *d, unsigned *mw)
{
    if (d != &dev0) return 2;
    if (getenv("FAKE_NVML_FAIL")) return 3; /* not supported */
    *mw = 123456;
    return 0;
}
