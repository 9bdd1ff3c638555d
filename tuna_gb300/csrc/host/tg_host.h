// tg_host.h — host-side pieces of libtuna_gpu.so: FASTA/FASTQ parsing into
// the sequence stream the kernels take, and the output writers.
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

// Output formatting of (key words, count) pairs.
struct Pairs {
    const uint64_t* keys;   // n * words
    const uint32_t* counts; // n
    uint64_t n;
    int words;
    int k;
};

// TSV lines "<kmer>\t<count>\n" for pairs [first, first + n), appended to out.
void format_tsv(const Pairs& p, uint64_t first, uint64_t n, std::string& out);
// KFF raw-section entries: ceil(k/4) bytes MSB-first, then the count as u32 BE.
void format_kff_entries(const Pairs& p, uint64_t first, uint64_t n, std::string& out);
// RAW: words then u32 count per pair, little-endian, packed.
void format_raw(const Pairs& p, uint64_t first, uint64_t n, std::string& out);
// The KFF container around n entries (header + variables + raw section start),
// and its closing footer.
std::string kff_header(int k, uint64_t n);
std::string kff_footer();

// Format with several threads into chunks of about chunk_pairs pairs and hand
// them, in order, to sink (returns false to stop). fmt: 0 TSV, 1 KFF, 2 RAW.
bool format_parallel(const Pairs& p, int fmt, unsigned threads,
                     bool (*sink)(const std::string& chunk, uint64_t npairs, void* user), void* user);

}  // namespace tgh
