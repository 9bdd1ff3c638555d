// Stand-in for the kff-cpp-api header that the reference includes from
// src/kff_output.hpp. kff-cpp-api is fetched by the reference's CMake at
// configure time (no network here), so the reference is compiled against
// these declarations instead. They only let the TSV path link: any attempt
// to write KFF through them throws. KFF parity is pinned separately by
// decoding KFF files back to (k-mer, count) pairs.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>

struct Kff_file {
    Kff_file(const std::string&, const std::string&) { fail(); }
    void write_encoding(int, int, int, int) { fail(); }
    void set_uniqueness(bool) { fail(); }
    void set_canonicity(bool) { fail(); }
    void write_metadata(uint32_t, uint8_t*) { fail(); }
    [[noreturn]] static void fail() {
        throw std::runtime_error("KFF output is not available in this oracle build");
    }
};
struct Section_GV {
    explicit Section_GV(Kff_file*) { Kff_file::fail(); }
    void write_var(const std::string&, uint64_t) {}
    void close() {}
};
struct Section_Raw {
    explicit Section_Raw(Kff_file*) { Kff_file::fail(); }
    void write_compacted_sequence(uint8_t*, uint64_t, uint8_t*) {}
    void close() {}
};
