// No-op stand-in for HighFive's H5Easy (FRICO only writes optional dumps).
#pragma once
#include <string>
namespace H5Easy {
struct File {
    enum Mode { Truncate };
    File(const std::string&, Mode) {}
    template <typename T> void createDataSet(const std::string&, const T&) {}
};
}  // namespace H5Easy
