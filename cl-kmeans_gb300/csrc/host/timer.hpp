// Host wall-clock timer (timer.hpp:48-66 of the reference): steady_clock.
#pragma once

#include <chrono>
#include <cstdint>

namespace Timer {

class Timer {
public:
    void start() { begin_ = std::chrono::steady_clock::now(); }
    template <typename Duration>
    uint64_t stop() {
        auto end = std::chrono::steady_clock::now();
        return (uint64_t)std::chrono::duration_cast<Duration>(end - begin_).count();
    }

private:
    std::chrono::steady_clock::time_point begin_;
};

}  // namespace Timer
