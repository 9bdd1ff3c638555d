// output.cpp — the KFF container around the entries the device formats
// (tg_format.cu): the header and footer the reference writes through
// kff-cpp-api (src/kff_output.hpp:20-57): encoding A0 C1 G2 T3, unique and
// canonical flags, variables k, max = 1, data_size = 4, one raw section.
#include "tg_host.h"

#include <cstring>

namespace tgh {

static void put_be(std::string& s, uint64_t v, int n) {
    for (int i = n - 1; i >= 0; --i) s.push_back((char)((v >> (8 * i)) & 0xFF));
}
static void put_var(std::string& s, const char* name, uint64_t v) {
    s.append(name, strlen(name) + 1);
    put_be(s, v, 8);
}

std::string kff_header(int k, uint64_t n) {
    std::string s;
    s.append("KFF", 3);
    s.push_back(1);
    s.push_back(0);
    s.push_back((char)0x1B);  // A=00 C=01 G=10 T=11
    s.push_back(1);           // unique
    s.push_back(1);           // canonical
    put_be(s, 0, 4);          // no metadata
    s.push_back('v');
    put_be(s, 3, 8);
    put_var(s, "k", (uint64_t)k);
    put_var(s, "max", 1);
    put_var(s, "data_size", 4);
    s.push_back('r');
    put_be(s, n, 8);
    return s;
}

std::string kff_footer() {
    std::string s;
    const char* nm = "footer_size";
    const uint64_t fsz = 1 + 8 + strlen(nm) + 1 + 8 + 3;
    s.push_back('v');
    put_be(s, 1, 8);
    put_var(s, nm, fsz);
    s.append("KFF", 3);
    return s;
}

}  // namespace tgh
