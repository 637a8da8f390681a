// Minimal test harness for the C++ façade tests: CHECK records failures,
// CHECK_THROWS_AS checks the exception type, main returns the failure count.
#pragma once
#include <cmath>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

namespace check {
inline int& failures() { static int f = 0; return f; }
inline std::vector<std::pair<const char*, std::function<void()>>>& cases() {
    static std::vector<std::pair<const char*, std::function<void()>>> c;
    return c;
}
struct Reg {
    Reg(const char* name, std::function<void()> fn) { cases().emplace_back(name, std::move(fn)); }
};
inline bool approx(double a, double b, double rel) { return std::fabs(a - b) <= rel * std::fmax(std::fabs(b), 1e-30); }
inline int run_all() {
    for (auto& c : cases()) {
        const int before = failures();
        try {
            c.second();
        } catch (const std::exception& e) {
            std::printf("  unexpected exception: %s\n", e.what());
            ++failures();
        }
        std::printf("%s %s\n", failures() == before ? "PASS" : "FAIL", c.first);
    }
    std::printf("%d failure(s)\n", failures());
    return failures() ? 1 : 0;
}
}  // namespace check

#define CHECK_CAT2(a, b) a##b
#define CHECK_CAT(a, b) CHECK_CAT2(a, b)
#define TEST_CASE(name)                                                     \
    static void CHECK_CAT(test_fn_, __LINE__)();                            \
    static check::Reg CHECK_CAT(test_reg_, __LINE__)(name, CHECK_CAT(test_fn_, __LINE__)); \
    static void CHECK_CAT(test_fn_, __LINE__)()
#define CHECK(cond)                                                         \
    do {                                                                    \
        if (!(cond)) {                                                      \
            std::printf("  %s:%d: CHECK(%s) failed\n", __FILE__, __LINE__, #cond); \
            ++check::failures();                                            \
        }                                                                   \
    } while (0)
#define CHECK_THROWS_AS(expr, type)                                         \
    do {                                                                    \
        bool ok_ = false;                                                   \
        try { (void)(expr); } catch (const type&) { ok_ = true; } catch (...) {} \
        if (!ok_) {                                                         \
            std::printf("  %s:%d: %s did not throw %s\n", __FILE__, __LINE__, #expr, #type); \
            ++check::failures();                                            \
        }                                                                   \
    } while (0)
