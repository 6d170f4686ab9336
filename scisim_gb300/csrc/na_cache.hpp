// na_cache.hpp -- per-device cache of a device address that belongs to one CUDA context.
//
// The allocation-free solve keeps its scratch in a file-scope __device__ array; host code must
// pass that array's device address, which cudaGetSymbolAddress looks up in the context current on
// the device.  A context that is torn down and created again (cudaDeviceReset, or another runtime
// releasing the primary context) loads the module again, possibly at another address, so a cached
// address is only valid together with the identity of the context it was looked up in.  This
// cache keys each device's entry on that identity (a per-process unique context id), looks the
// address up again whenever the current context differs, and serialises the look-up and update of
// an entry with a mutex so that host threads calling at the same time see a matching pair.  It has
// no CUDA dependency so that its logic can be tested on a machine without a GPU.
#pragma once

#include <mutex>

namespace sg {

template <int kDevices>
class DeviceAddressCache {
 public:
  // The address for device `dev` in its current context.  current_id(&id) returns false or
  // id = 0 when the context's identity is unknown (no context current yet, or no driver entry
  // point): then the address is looked up and nothing is cached.  lookup(&addr) returns a status
  // (0 = success) and may make the device's context current, so the identity is read again after
  // it.  Returns lookup's status, or -1 for a device outside [0, kDevices).
  template <class CurrentId, class Lookup>
  int get(int dev, CurrentId current_id, Lookup lookup, void** out) {
    if (dev < 0 || dev >= kDevices) return -1;
    std::lock_guard<std::mutex> lock(m_mutex[dev]);
    unsigned long long id = 0;
    if (current_id(&id) && id != 0 && id == m_id[dev] && m_addr[dev] != nullptr) {
      *out = m_addr[dev];
      return 0;
    }
    void* addr = nullptr;
    const int status = lookup(&addr);
    if (status != 0) return status;
    unsigned long long after = 0;
    if (current_id(&after) && after != 0) {
      m_id[dev] = after;
      m_addr[dev] = addr;
    } else {
      m_id[dev] = 0;
      m_addr[dev] = nullptr;
    }
    *out = addr;
    return 0;
  }

 private:
  std::mutex m_mutex[kDevices];
  unsigned long long m_id[kDevices] = {};
  void* m_addr[kDevices] = {};
};

}  // namespace sg
