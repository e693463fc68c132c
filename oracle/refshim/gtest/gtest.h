// Minimal stand-in for the handful of googletest macros a plain unit-test
// file needs (TEST, EXPECT_EQ/TRUE/FALSE, InitGoogleTest, RUN_ALL_TESTS), so
// such a file builds against the oracle without googletest installed.
// Test infrastructure only.
#pragma once

#include <cstdio>
#include <functional>
#include <sstream>
#include <string>
#include <vector>

namespace testing {

struct Case
{
  std::string suite, name;
  std::function<void()> body;
};

inline std::vector<Case>& registry()
{
  static std::vector<Case> r;
  return r;
}

inline int& failures()
{
  static int f = 0;
  return f;
}

struct Registrar
{
  Registrar(const char* suite, const char* name, void (*fn)())
  {
    registry().push_back(Case{suite, name, fn});
  }
};

template <class A, class B>
inline void expect_eq(const A& a, const B& b, const char* ea, const char* eb, const char* file, int line)
{
  if (!(a == b))
  {
    std::ostringstream os;
    os.precision(17);
    os << file << ":" << line << ": EXPECT_EQ(" << ea << ", " << eb << ") failed: " << a << " vs " << b;
    std::fprintf(stderr, "%s\n", os.str().c_str());
    ++failures();
  }
}

inline void expect_bool(bool v, bool want, const char* e, const char* file, int line)
{
  if (v != want)
  {
    std::fprintf(stderr, "%s:%d: EXPECT_%s(%s) failed\n", file, line, want ? "TRUE" : "FALSE", e);
    ++failures();
  }
}

inline void InitGoogleTest(int*, char**) {}

inline int run_all()
{
  int failed_cases = 0;
  for (const Case& c : registry())
  {
    const int before = failures();
    c.body();
    const bool ok = failures() == before;
    std::printf("[%s] %s.%s\n", ok ? "       OK " : "  FAILED  ", c.suite.c_str(), c.name.c_str());
    if (!ok) ++failed_cases;
  }
  std::printf("%zu tests, %d failed\n", registry().size(), failed_cases);
  return failed_cases == 0 ? 0 : 1;
}

} // namespace testing

#define TEST(suite, name)                                                                      \
  static void suite##_##name##_body();                                                         \
  static ::testing::Registrar suite##_##name##_registrar(#suite, #name, &suite##_##name##_body); \
  static void suite##_##name##_body()

#define EXPECT_EQ(a, b) ::testing::expect_eq((a), (b), #a, #b, __FILE__, __LINE__)
#define EXPECT_TRUE(c) ::testing::expect_bool(static_cast<bool>(c), true, #c, __FILE__, __LINE__)
#define EXPECT_FALSE(c) ::testing::expect_bool(static_cast<bool>(c), false, #c, __FILE__, __LINE__)
#define RUN_ALL_TESTS() ::testing::run_all()
