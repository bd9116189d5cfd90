// Per-device one-time set-up, for state that the CUDA runtime keeps per
// device: kernel attributes set by cudaFuncSetAttribute, occupancy figures
// measured on a device, the device address of a __device__ array.  Each
// device that a thread makes current runs the set-up once, with that device
// current; a set-up that fails is not recorded, so the next call retries it.
//
// Host-only and free of CUDA headers, so that the bookkeeping can be
// compiled and tested without a GPU.
#ifndef LPMA_PER_DEVICE_H
#define LPMA_PER_DEVICE_H

#include <mutex>

namespace lpma {

constexpr int MAX_DEVICES = 64;

// T: what the set-up produces for one device (e.g. an occupancy table).
template <typename T>
class PerDevice {
public:
    // Runs setup(dev, value) the first time `dev` asks (setup returns 0 on
    // success, any other value is passed back and nothing is recorded);
    // afterwards returns 0 and leaves *out pointing at the device's value.
    // A device id outside [0, MAX_DEVICES) returns `bad_device`.
    template <typename F>
    int get(int dev, F &&setup, const T **out, int bad_device) {
        if (dev < 0 || dev >= MAX_DEVICES) return bad_device;
        std::lock_guard<std::mutex> lk(mu_);
        if (!done_[dev]) {
            T v{};
            const int e = setup(dev, v);
            if (e) return e;
            value_[dev] = v;
            done_[dev] = true;
        }
        if (out) *out = &value_[dev];
        return 0;
    }

    // the recorded value of a device that finished its set-up, else nullptr
    const T *peek(int dev) const {
        if (dev < 0 || dev >= MAX_DEVICES) return nullptr;
        std::lock_guard<std::mutex> lk(mu_);
        return done_[dev] ? &value_[dev] : nullptr;
    }

private:
    mutable std::mutex mu_;
    bool done_[MAX_DEVICES] = {};
    T value_[MAX_DEVICES] = {};
};

}  // namespace lpma

#endif
