// fatal.cuh -- structured fatal errors raised inside the library.
//
// Internal code throws FatalError; every extern "C" entry point catches it,
// records the code and detail (ppf_fatal_code / ppf_fatal_detail) and then
// either exits with status 1, as the reference does (main/fatal.hpp), or --
// when the host sets PPF_RETURN_ON_FATAL=1 -- returns a failed result so an
// in-process harness survives.
#pragma once

#include <exception>
#include <string>

extern "C" {
extern unsigned char g_ppf_fatal_code;
extern char g_ppf_fatal_detail[512];
}

namespace ppf {

struct FatalError : std::exception {
    unsigned char code;
    std::string detail;
    FatalError(unsigned char c, std::string d) : code(c), detail(std::move(d)) {}
    const char *what() const noexcept override { return detail.c_str(); }
};

void set_fatal(unsigned char code, const char *detail);

} // namespace ppf
