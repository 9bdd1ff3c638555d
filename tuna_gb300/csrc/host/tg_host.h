// tg_host.h — host-side pieces of libtuna_gpu.so: input files, the host
// FASTA/FASTQ parser (the reference's rules; the device lexer hands it the
// files it flags) and the KFF container.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace tgh {

// Append the ACGT runs of a FASTA/FASTQ buffer to out, each followed by one
// separator byte ('\n'). FASTQ iff data[0] == '@'. Follows the reference's
// parser (include/helicase_cpp/parser_fasta.hpp, parser_fastq.hpp). Returns
// false for an empty buffer ("Empty file").
bool fastx_to_stream(const uint8_t* data, size_t len, std::vector<uint8_t>& out);

// Read a whole file, inflating gzip when the name ends in ".gz" (the choice of
// src/seq_source.hpp:196-204). Returns an error message, or "" on success.
std::string read_input_file(const std::string& path, std::vector<uint8_t>& out);

// The KFF container around n entries (header + variables + raw section start),
// and its closing footer.
std::string kff_header(int k, uint64_t n);
std::string kff_footer();

}  // namespace tgh
