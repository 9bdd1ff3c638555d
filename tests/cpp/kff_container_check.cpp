// kff_container_check.cpp — the KFF header and footer the library writes
// around the device-formatted entries (tgh::kff_header / kff_footer in
// csrc/host/output.cpp), without a GPU: `kff_container_check k n out` writes
// the header for k and n entries to out.head and the footer to out.foot.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "host/tg_host.h"

static bool write_file(const std::string& path, const std::string& bytes) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    return std::fclose(f) == 0 && ok;
}

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    const int k = std::atoi(argv[1]);
    const unsigned long long n = std::strtoull(argv[2], nullptr, 10);
    const std::string out = argv[3];
    return write_file(out + ".head", tgh::kff_header(k, n)) && write_file(out + ".foot", tgh::kff_footer()) ? 0 : 1;
}
