// A small stand-in for the Catch2 macros the reference's test scenarios use,
// so that those scenario files compile unchanged against the C++ façade
// (include/stpgb.hpp).  Every GIVEN / WHEN / THEN block runs once, in source
// order: enough for scenarios whose blocks only read values.  main() runs
// every scenario and returns the number of failed checks.
#pragma once
#include <cstdio>
#include <functional>
#include <vector>

namespace stpgb_catch {

inline std::vector<std::pair<const char*, std::function<void()>>>& scenarios() {
	static std::vector<std::pair<const char*, std::function<void()>>> all;
	return all;
}

inline int& failures() {
	static int n = 0;
	return n;
}

struct Registrar {
	Registrar(const char* name, void (*f)()) {
		scenarios().emplace_back(name, f);
	}
};

inline void check(const bool ok, const char* expr, const char* file, const int line) {
	if (!ok) {
		std::printf("%s:%d: check failed: %s\n", file, line, expr);
		failures()++;
	}
}

} // namespace stpgb_catch

#define STPGB_CATCH_CAT2(a, b) a##b
#define STPGB_CATCH_CAT(a, b) STPGB_CATCH_CAT2(a, b)
#define SCENARIO(name, ...) \
	static void STPGB_CATCH_CAT(stpgb_scenario_, __LINE__)(); \
	static const stpgb_catch::Registrar STPGB_CATCH_CAT(stpgb_registrar_, __LINE__)(name, \
		&STPGB_CATCH_CAT(stpgb_scenario_, __LINE__)); \
	static void STPGB_CATCH_CAT(stpgb_scenario_, __LINE__)()
#define GIVEN(...) if (true)
#define AND_GIVEN(...) if (true)
#define WHEN(...) if (true)
#define AND_WHEN(...) if (true)
#define THEN(...) if (true)
#define AND_THEN(...) if (true)
#define CHECK(...) stpgb_catch::check(static_cast<bool>(__VA_ARGS__), #__VA_ARGS__, __FILE__, __LINE__)
#define CHECK_FALSE(...) stpgb_catch::check(!static_cast<bool>(__VA_ARGS__), "!(" #__VA_ARGS__ ")", __FILE__, __LINE__)
#define REQUIRE(...) CHECK(__VA_ARGS__)

#ifdef STPGB_CATCH_MAIN
int main() {
	for (const auto& s : stpgb_catch::scenarios()) {
		std::printf("scenario: %s\n", s.first);
		s.second();
	}
	std::printf("%zu scenarios, %d failed checks\n", stpgb_catch::scenarios().size(), stpgb_catch::failures());
	return stpgb_catch::failures() == 0 && !stpgb_catch::scenarios().empty() ? 0 : 1;
}
#endif
