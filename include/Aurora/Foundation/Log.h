// Logging macros and the Log singleton that Aurora's public header refers to, for builds of the
// GB300 backend's Aurora interface without Aurora's Foundation library.  Messages go to stderr;
// AU_FAIL (and a failed AU_ASSERT) aborts, as Foundation's default does.  Programs that link
// Foundation itself use its Log.h instead; the backend's own code does not depend on this class.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <string>

namespace Aurora
{
namespace Foundation
{

class Log
{
public:
    enum class Level
    {
        kInfo,
        kWarn,
        kError,
        kFail
    };

    template <typename... Args>
    static bool report(Level level, const char* file, int line, const std::string& format, Args... args)
    {
        static const char* tag[] = { "info", "warning", "error", "failure" };
        std::fprintf(stderr, "Aurora %s (%s:%d): ", tag[int(level)], file, line);
        if constexpr (sizeof...(Args) > 0)
            std::fprintf(stderr, format.c_str(), args...);
        else
            std::fputs(format.c_str(), stderr);
        std::fputc('\n', stderr);
        if (level == Level::kFail)
            std::abort();
        return true;
    }
};

} // namespace Foundation
} // namespace Aurora

#define AU_INFO(_msg, ...) Aurora::Foundation::Log::report(Aurora::Foundation::Log::Level::kInfo, __FILE__, __LINE__, _msg, ##__VA_ARGS__)
#define AU_WARN(_msg, ...) Aurora::Foundation::Log::report(Aurora::Foundation::Log::Level::kWarn, __FILE__, __LINE__, _msg, ##__VA_ARGS__)
#define AU_ERROR(_msg, ...) Aurora::Foundation::Log::report(Aurora::Foundation::Log::Level::kError, __FILE__, __LINE__, _msg, ##__VA_ARGS__)
#define AU_FAIL(_msg, ...) Aurora::Foundation::Log::report(Aurora::Foundation::Log::Level::kFail, __FILE__, __LINE__, _msg, ##__VA_ARGS__)
#define AU_ASSERT(_check, _msg, ...)                                                               \
    do                                                                                             \
    {                                                                                              \
        if (!(_check))                                                                             \
            AU_FAIL("assertion failed: %s: " _msg, #_check, ##__VA_ARGS__);                        \
    } while (0)
