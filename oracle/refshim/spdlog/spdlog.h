// Minimal no-op logging shim so the reference renderer's sources compile
// without their (unvendored) logging dependency. Every call is discarded:
// the shim carries no arithmetic and does not change any rendered value.
#pragma once
#include <chrono>

namespace spdlog
{
namespace level
{
enum level_enum { trace, debug, info, warn, err, critical, off };
}

template <typename... Args> inline void trace(Args&&...) {}
template <typename... Args> inline void debug(Args&&...) {}
template <typename... Args> inline void info(Args&&...) {}
template <typename... Args> inline void warn(Args&&...) {}
template <typename... Args> inline void error(Args&&...) {}
inline void set_pattern(const char*) {}
inline void set_level(level::level_enum) {}

// Wall-clock stopwatch with the two members the renderer calls.
class stopwatch
{
public:
    stopwatch() : m_start(std::chrono::steady_clock::now()) {}
    void reset() { m_start = std::chrono::steady_clock::now(); }
    double elapsed() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - m_start).count();
    }

private:
    std::chrono::steady_clock::time_point m_start;
};
}  // namespace spdlog
