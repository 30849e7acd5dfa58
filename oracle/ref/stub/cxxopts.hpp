// cxxopts.hpp -- a stand-in for the command-line library that the reference's
// examples/spmv/helpers.hxx includes.  helpers.hxx uses it only in its
// parameters_t struct (command-line parsing), which oracle/ref/ref_cpu.cu
// never constructs; these declarations exist so that the header compiles.
// Nothing here parses anything.  Test infrastructure only.
#pragma once

#include <cstddef>
#include <initializer_list>
#include <memory>
#include <string>

namespace cxxopts {

struct value_base {};

template <class T>
std::shared_ptr<value_base> value() {
  return nullptr;
}

struct OptionAdder {
  OptionAdder& operator()(const std::string&, const std::string&,
                          std::shared_ptr<value_base> = nullptr) {
    return *this;
  }
};

struct OptionValue {
  template <class T>
  const T& as() const {
    static const T t{};
    return t;
  }
};

struct ParseResult {
  std::size_t count(const std::string&) const { return 0; }
  const OptionValue& operator[](const std::string&) const {
    static const OptionValue v;
    return v;
  }
};

struct Options {
  Options(std::string, std::string) {}
  OptionAdder add_options(std::string = "") { return OptionAdder(); }
  ParseResult parse(int, char**) { return ParseResult(); }
  std::string help(std::initializer_list<std::string> = {}) const { return std::string(); }
};

}  // namespace cxxopts
