// Drives the C++ counting API (include/tuna/tuna.hpp) the way a user of the
// reference's tuna.hpp would, and prints "<kmer>\t<count>" lines (any order).
//   api_check <k> <m> <mode> <min_count> <max_count> <file>...
//   mode: count_to | raw | cb_ascii | cb_binary
// Exit codes: 0 ok, 2 usage, 3 std::invalid_argument, 4 std::runtime_error.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "tuna/tuna.hpp"

namespace {

template <uint16_t k, uint16_t m>
int run(const std::string& mode, const tuna::Options& o, const std::vector<std::string>& files) {
    std::string out;
    auto line = [&](std::string_view km, uint32_t c) {
        out.append(km);
        out.push_back('\t');
        out.append(std::to_string(c));
        out.push_back('\n');
    };
    if (mode == "count_to") {
        for (const auto& kv : tuna::count_to<k, m>(files, o)) line(kv.first, kv.second);
    } else if (mode == "raw") {
        for (const auto& kv : tuna::count_to_raw<k, m>(files, o)) line(kv.first.string_label(), kv.second);
    } else if (mode == "cb_ascii") {
        tuna::count<k, m>(files, [&](std::string_view km, uint32_t c) { line(km, c); }, o);
    } else if (mode == "cb_binary") {
        tuna::count<k, m>(files, [&](const tuna::Kmer<k>& km, uint32_t c) { line(km.string_label(), c); }, o);
    } else {
        return 2;
    }
    fwrite(out.data(), 1, out.size(), stdout);
    return 0;
}

using Fn = int (*)(const std::string&, const tuna::Options&, const std::vector<std::string>&);
struct Entry {
    int k, m;
    Fn fn;
};
const Entry kTable[] = {
    {31, 21, run<31, 21>}, {31, 23, run<31, 23>}, {15, 9, run<15, 9>},  {5, 3, run<5, 3>},
    {9, 5, run<9, 5>},     {21, 17, run<21, 17>}, {25, 21, run<25, 21>}, {33, 21, run<33, 21>},
    {63, 21, run<63, 21>},
};

}  // namespace

int main(int argc, char** argv) {
    if (argc < 6) return 2;
    const int k = atoi(argv[1]), m = atoi(argv[2]);
    const std::string mode = argv[3];
    tuna::Options o;
    o.min_count = (uint32_t)strtoul(argv[4], nullptr, 10);
    o.max_count = (uint32_t)strtoul(argv[5], nullptr, 10);
    std::vector<std::string> files(argv + 6, argv + argc);
    try {
        for (const Entry& e : kTable)
            if (e.k == k && e.m == m) return e.fn(mode, o, files);
        return 2;
    } catch (const std::invalid_argument& e) {
        std::cerr << "invalid_argument: " << e.what() << "\n";
        return 3;
    } catch (const std::runtime_error& e) {
        std::cerr << "runtime_error: " << e.what() << "\n";
        return 4;
    }
}
