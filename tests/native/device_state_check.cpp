// Host-side check of the per-device set-up bookkeeping (gpe_device_state.h):
// set-up runs once per device, not once per process; a failed set-up is
// retried; out-of-range ordinals are refused; concurrent first calls from
// several threads leave every device configured with the same value.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "gpe_device_state.h"

#define CHECK(c)                                                      \
    do {                                                              \
        if (!(c)) {                                                   \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            return 1;                                                 \
        }                                                             \
    } while (0)

int main() {
    using gpe::DeviceOnce;
    using gpe::DeviceValue;
    constexpr int kBad = -77;

    // configured on device 0 does not mean configured on device 1
    DeviceOnce once;
    int runs[gpe::kMaxDevices] = {0};
    auto setup_for = [&](int d) { return [&, d] { runs[d]++; return 0; }; };
    CHECK(once.ensure(0, setup_for(0), kBad) == 0);
    CHECK(once.done(0) && !once.done(1));
    CHECK(once.ensure(0, setup_for(0), kBad) == 0);
    CHECK(runs[0] == 1);
    CHECK(once.ensure(1, setup_for(1), kBad) == 0);
    CHECK(runs[1] == 1 && once.done(1));
    CHECK(once.ensure(63, setup_for(63), kBad) == 0 && once.done(63));

    // a failed set-up is not recorded and is retried on the next call
    int fails = 0;
    CHECK(once.ensure(5, [&] { fails++; return 42; }, kBad) == 42);
    CHECK(!once.done(5));
    CHECK(once.ensure(5, [&] { fails++; return 0; }, kBad) == 0);
    CHECK(fails == 2 && once.done(5));

    // ordinals outside the table are refused without running the set-up
    CHECK(once.ensure(-1, [&] { fails++; return 0; }, kBad) == kBad);
    CHECK(once.ensure(gpe::kMaxDevices, [&] { fails++; return 0; }, kBad) == kBad);
    CHECK(fails == 2 && !once.done(-1) && !once.done(gpe::kMaxDevices));

    // per-device values: computed once per device, each device its own
    DeviceValue<unsigned> val;
    unsigned v = 0;
    int computes = 0;
    CHECK(val.ensure(2, &v, [&](unsigned* o) { computes++; *o = 152u * 7u; return 0; }, kBad) == 0);
    CHECK(v == 1064u && val.get(2) == 1064u && val.get(3) == 0u);
    CHECK(val.ensure(2, &v, [&](unsigned* o) { computes++; *o = 1u; return 0; }, kBad) == 0);
    CHECK(v == 1064u && computes == 1);
    CHECK(val.ensure(3, &v, [&](unsigned* o) { computes++; *o = 132u; return 0; }, kBad) == 0);
    CHECK(v == 132u && val.get(2) == 1064u && computes == 2);
    CHECK(val.ensure(70, &v, [&](unsigned* o) { *o = 9u; return 0; }, kBad) == kBad);
    CHECK(val.ensure(4, &v, [&](unsigned* o) { *o = 9u; return 7; }, kBad) == 7 && val.get(4) == 0u);

    // many threads making their first call on the same devices at once
    DeviceOnce shared;
    DeviceValue<void*> addr;
    std::atomic<int> setups{0};
    static int anchor[8];
    std::vector<std::thread> pool;
    for (int t = 0; t < 16; t++) {
        pool.emplace_back([&, t] {
            const int d = t % 8;
            for (int k = 0; k < 1000; k++) {
                if (shared.ensure(d, [&] { setups++; return 0; }, kBad) != 0) std::abort();
                void* p = nullptr;
                if (addr.ensure(d, &p, [&](void** o) { *o = &anchor[d]; return 0; }, kBad) != 0) std::abort();
                if (p != &anchor[d]) std::abort();
            }
        });
    }
    for (auto& th : pool) th.join();
    for (int d = 0; d < 8; d++) CHECK(shared.done(d) && addr.get(d) == &anchor[d]);
    CHECK(!shared.done(8));
    CHECK(setups.load() >= 8 && setups.load() <= 16);  // at most one per racing thread and device
    std::printf("device state ok\n");
    return 0;
}
