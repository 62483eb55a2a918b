// Self-test of the bounded device-side wait: a cooperative kernel in which
// block 0 never arrives at the grid barrier, so every other block's wait runs
// into the timeout and the kernel reports IG_ERR_TIMEOUT through the control
// block.  The wait is bounded by %globaltimer; nothing faults or hangs.
#include "ig_device.cuh"

namespace {
__global__ void selftest_missing_arrival(IgCtl* ctl, unsigned long long timeout_ns) {
  if (blockIdx.x == 0) return;  // the arrival that never comes
  if (!ig::grid_sync(ctl, timeout_ns)) return;
  if (threadIdx.x == 0) atomicAdd(&ctl->i32[0], 1);  // not reached when the barrier fails
}
}  // namespace

extern "C" int ig_selftest_wait_timeout(int timeout_ms, int* observed_status) {
  if (timeout_ms < 1 || !observed_status) return ig_fail(IG_ERR_INVALID_ARG, "bad argument");
  IgDevice* dev = nullptr;
  int rc = ig_current_device(&dev);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(dev->mu);
  IgExec ex;
  if ((rc = ig_exec_init(&ex, dev->stream, &dev->scratch, dev->h_ctl, dev->id, dev->sms))) return rc;
  ex.timeout_ns = (unsigned long long)timeout_ms * 1000000ull;
  if ((rc = ig_exec_reset(&ex))) return rc;
  unsigned long long t = ex.timeout_ns;
  void* args[] = {&ex.d_ctl, &t};
  if ((rc = ig_launch_coop(&ex, (const void*)selftest_missing_arrival, 64, 0, 1, args, nullptr))) return rc;
  *observed_status = ig_exec_finish(&ex);
  ig_clear_error();
  return IG_OK;
}
