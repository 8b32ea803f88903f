// Golden strings for frico_gb300.outputs.cpp_format: std::format("{}", x) for
// the doubles listed (as C99 hex floats, exact) on standard input, one per line.
// Output: "<hex> <formatted>" per line.
#include <cstdio>
#include <cstdlib>
#include <format>
#include <string>

int main() {
    char buf[128];
    while (std::fgets(buf, sizeof buf, stdin)) {
        std::string s(buf);
        while (!s.empty() && (s.back() == '\n' || s.back() == '\r')) s.pop_back();
        if (s.empty()) continue;
        double x = std::strtod(s.c_str(), nullptr);
        std::printf("%s %s\n", s.c_str(), std::format("{}", x).c_str());
    }
    return 0;
}
