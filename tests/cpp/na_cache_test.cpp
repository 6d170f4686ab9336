// Test of the per-context device-address cache of the allocation-free solve
// (scisim_gb300/csrc/na_cache.hpp), run on the CPU with stand-ins for the context identity and the
// symbol look-up.  Exit status 0 = pass.
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "../../scisim_gb300/csrc/na_cache.hpp"

namespace {

int fail(const char* what) {
  std::fprintf(stderr, "FAILED: %s\n", what);
  return EXIT_FAILURE;
}

}  // namespace

int main() {
  sg::DeviceAddressCache<4> cache;
  unsigned long long ctx_id = 0;  // the "current context" (0: none yet)
  int lookups = 0;
  char module_a[16], module_b[16];
  void* module = module_a;  // where the "module" of the current context is loaded
  auto current = [&](unsigned long long* id) {
    *id = ctx_id;
    return ctx_id != 0;
  };
  auto lookup = [&](void** addr) {
    ++lookups;
    if (ctx_id == 0) ctx_id = 7;  // the look-up initialises the device's primary context
    *addr = module;
    return 0;
  };
  void* p = nullptr;
  // First call: no context yet; the look-up creates one and its identity is recorded after it.
  if (cache.get(0, current, lookup, &p) != 0 || p != module_a || lookups != 1) return fail("first look-up");
  // Same context: served from the cache.
  if (cache.get(0, current, lookup, &p) != 0 || p != module_a || lookups != 1) return fail("cached");
  // The context is torn down and created again (cudaDeviceReset): the module moves.
  ctx_id = 8;
  module = module_b;
  if (cache.get(0, current, lookup, &p) != 0 || p != module_b || lookups != 2) return fail("after a new context");
  if (cache.get(0, current, lookup, &p) != 0 || p != module_b || lookups != 2) return fail("cached again");
  // Devices have entries of their own.
  if (cache.get(1, current, lookup, &p) != 0 || p != module_b || lookups != 3) return fail("second device");
  if (cache.get(4, current, lookup, &p) != -1 || cache.get(-1, current, lookup, &p) != -1) return fail("range");
  // Unknown identity: looked up every time, nothing cached.
  auto unknown = [](unsigned long long* id) {
    *id = 0;
    return false;
  };
  const int before = lookups;
  cache.get(2, unknown, lookup, &p);
  cache.get(2, unknown, lookup, &p);
  if (lookups != before + 2) return fail("unknown identity is not cached");
  // A failed look-up returns its status and leaves the entry untouched.
  auto failing = [](void**) { return 4; };
  ctx_id = 9;
  if (cache.get(0, current, failing, &p) != 4) return fail("look-up status");
  // Concurrent callers on one device all get the address of the current context.
  ctx_id = 10;
  module = module_a;
  std::vector<std::thread> ts;
  std::vector<void*> got(8, nullptr);
  for (int t = 0; t < 8; ++t)
    ts.emplace_back([&, t] {
      for (int k = 0; k < 1000; ++k) cache.get(3, current, lookup, &got[t]);
    });
  for (std::thread& t : ts) t.join();
  for (void* g : got)
    if (g != module_a) return fail("threads");
  return EXIT_SUCCESS;
}
