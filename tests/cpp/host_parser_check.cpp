// host_parser_check.cpp — the library's host FASTA/FASTQ parser
// (tgh::fastx_to_stream in csrc/host/fastx.cpp, the path taken by the FASTQ
// files the device lexer hands back), run without a GPU: each input file named
// on the command line is read as the library reads it and its sequence stream
// is written to <file>.stream ("<file>.err" holds the message of a file that
// does not parse).
#include <cstdio>
#include <string>
#include <vector>

#include "host/tg_host.h"

static bool write_file(const std::string& path, const void* data, size_t n) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data, 1, n, f) == n;
    return std::fclose(f) == 0 && ok;
}

int main(int argc, char** argv) {
    for (int i = 1; i < argc; ++i) {
        const std::string path = argv[i];
        tgh::Bytes raw;
        std::string err = tgh::read_input_file(path, raw, 2);
        std::vector<uint8_t> out;
        if (err.empty() && !tgh::fastx_to_stream(raw.data(), raw.size(), out)) err = "Empty file";
        const bool ok = err.empty() ? write_file(path + ".stream", out.data(), out.size())
                                    : write_file(path + ".err", err.data(), err.size());
        if (!ok) {
            std::fprintf(stderr, "cannot write the output of %s\n", path.c_str());
            return 1;
        }
    }
    return 0;
}
