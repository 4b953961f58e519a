// device_session.cpp -- creation and release of the CUDA context beside host
// work, for a process that owns its device (the ngia2 command line).
//
// A CUDA process pays a fixed cost on each side of its device work: driver
// initialisation plus primary-context creation before the first call, and the
// context's teardown when it ends (about 0.2 s each on a GB300 host).  The
// reference pays both in every `-m clustering` run.  The command line starts
// the context on a helper thread while the host reads and indexes its input,
// and releases it (cudaDeviceReset) on a helper thread while the host writes
// its files, so only what the host work cannot cover stays on the clock.
// Library callers that share the device with other code never use these.
#include <cuda_runtime.h>

#include <thread>

#include "host.hpp"

namespace ngia {

namespace {
std::thread g_warmup, g_release;
int g_warmup_status = NGIA_OK, g_release_status = NGIA_OK;
}  // namespace

void device_warmup_start(int device) {
  if (g_warmup.joinable()) return;
  g_warmup = std::thread([device] {
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaFree(nullptr);  // creates the primary context
    g_warmup_status = e == cudaSuccess ? NGIA_OK : NGIA_ERR_CUDA;
  });
}

int device_warmup_join() {
  if (g_warmup.joinable()) g_warmup.join();
  return g_warmup_status;
}

void device_release_start(int device) {
  device_warmup_join();
  if (g_release.joinable()) return;
  g_release = std::thread([device] {
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceReset();
    g_release_status = e == cudaSuccess ? NGIA_OK : NGIA_ERR_CUDA;
  });
}

int device_release_join() {
  if (g_release.joinable()) g_release.join();
  return g_release_status;
}

}  // namespace ngia
