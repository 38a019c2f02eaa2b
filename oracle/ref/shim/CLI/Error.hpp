// Project-written stand-in for the one CLI11 type the reference's error header derives from
// (include/goofit/Error.h: struct GeneralError : CLI::Error).  CLI11 is an empty submodule of the
// reference; this shim is not a copy of it.
#pragma once
#include <stdexcept>
#include <string>

namespace CLI {
class Error : public std::runtime_error {
    int code_;
    std::string name_;

  public:
    Error(std::string name, std::string msg, int exit_code = 1)
        : std::runtime_error(msg), code_(exit_code), name_(std::move(name)) {}
    int get_exit_code() const { return code_; }
    std::string get_name() const { return name_; }
};
} // namespace CLI
