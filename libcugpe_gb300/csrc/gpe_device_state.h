// Per-device bookkeeping of one-time kernel set-up.
//
// Kernel attributes (the dynamic shared-memory opt-in, the carveout) and
// occupancy-derived figures belong to a device context, not to the process:
// a kernel configured on device 0 is not configured on device 1.  Each
// launcher therefore keeps one record per device ordinal.  Records are atomics
// so that host threads driving engines concurrently never race on them; two
// threads that configure the same device at the same time both run the
// (idempotent) set-up and publish the same value.
//
// Plain C++ with no CUDA dependency, so the bookkeeping is tested on the host.
#pragma once
#include <atomic>
#include <stdint.h>

namespace gpe {

constexpr int kMaxDevices = 64;

// One bit per device: set once the set-up of this object has succeeded on that device.
class DeviceOnce {
  public:
    bool done(int dev) const {
        return dev >= 0 && dev < kMaxDevices && ((bits_.load(std::memory_order_acquire) >> dev) & 1u);
    }
    // Runs `setup` (returning 0 on success) unless it already succeeded on `dev`; returns its result.
    // Device ordinals outside [0, kMaxDevices) are refused with `bad_device`.
    template <typename F>
    int ensure(int dev, F&& setup, int bad_device) {
        if (dev < 0 || dev >= kMaxDevices) return bad_device;
        if (done(dev)) return 0;
        const int rc = setup();
        if (rc == 0) bits_.fetch_or(uint64_t(1) << dev, std::memory_order_acq_rel);
        return rc;
    }

  private:
    std::atomic<uint64_t> bits_{0};
};

// One value per device (0 = not yet known).
template <typename T>
class DeviceValue {
  public:
    T get(int dev) const {
        return (dev >= 0 && dev < kMaxDevices) ? v_[dev].load(std::memory_order_acquire) : T(0);
    }
    // The value of `dev`, computed by `compute(T*)` (returning 0 on success) the first time.
    template <typename F>
    int ensure(int dev, T* out, F&& compute, int bad_device) {
        if (dev < 0 || dev >= kMaxDevices) return bad_device;
        T v = v_[dev].load(std::memory_order_acquire);
        if (v == T(0)) {
            const int rc = compute(&v);
            if (rc != 0) return rc;
            v_[dev].store(v, std::memory_order_release);
        }
        *out = v;
        return 0;
    }

  private:
    std::atomic<T> v_[kMaxDevices] = {};
};

}  // namespace gpe
