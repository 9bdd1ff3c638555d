// Exercises tuna::Kmer<k> (include/tuna/tuna.hpp) without a device: for each
// label on stdin prints the label read back, its reverse complement, its
// canonical form, the packed KFF bytes in hex, the words in hex and the
// comparisons with the previous label; the test checks them against Python.
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>

#include "tuna/tuna.hpp"

template <uint16_t k>
int run() {
    std::string line, prev;
    while (std::getline(std::cin, line)) {
        const tuna::Kmer<k> a(line);
        std::ostringstream os;
        os << a;
        uint8_t packed[(k + 3) / 4];
        a.write_packed_2bit_msb(packed);
        std::string hex;
        char b[8];
        for (uint8_t x : packed) {
            std::snprintf(b, sizeof b, "%02x", x);
            hex += b;
        }
        std::string words;
        for (uint16_t w = 0; w < tuna::Kmer<k>::num_words(); ++w) {
            char buf[24];
            std::snprintf(buf, sizeof buf, "%016llx", (unsigned long long)a.data()[w]);
            words += (w ? "," : "") + std::string(buf);
        }
        int cmp = 0;
        if (!prev.empty()) {
            const tuna::Kmer<k> p(prev.c_str());
            cmp = a < p ? -1 : (a > p ? 1 : 0);
            if ((cmp == 0) != (a == p) || (cmp != 0) != (a != p)) return 5;
        }
        std::cout << os.str() << " " << a.reverse_complement().string_label() << " "
                  << static_cast<std::string>(a.canonical()) << " " << hex << " " << words << " " << cmp << " "
                  << int(a.front()) << int(a.back()) << "\n";
        prev = line;
    }
    return 0;
}

int main(int argc, char** argv) {
    const int k = argc > 1 ? std::atoi(argv[1]) : 31;
    if (k == 31) return run<31>();
    if (k == 32) return run<32>();
    if (k == 63) return run<63>();
    if (k == 5) return run<5>();
    return 2;
}
