// tg_host.h — host-side pieces of libtuna_gpu.so: input files, the host
// FASTA/FASTQ parser (the reference's rules; the device lexer hands it the
// files it flags) and the KFF container.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <new>
#include <string>
#include <vector>

namespace tgh {

// A byte vector whose resize leaves new bytes uninitialised (input files are
// read or inflated straight into it, by several threads for BGZF).
template <typename T>
struct NoInitAlloc : std::allocator<T> {
    template <typename U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <typename U>
    NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    template <typename U>
    void construct(U* p) noexcept {
        ::new (static_cast<void*>(p)) U;
    }
    template <typename U, typename... Args>
    void construct(U* p, Args&&... args) {
        ::new (static_cast<void*>(p)) U(static_cast<Args&&>(args)...);
    }
};
using Bytes = std::vector<uint8_t, NoInitAlloc<uint8_t>>;

// Append the ACGT runs of a FASTA/FASTQ buffer to out, each followed by one
// separator byte ('\n'). FASTQ iff data[0] == '@'. Follows the reference's
// parser (include/helicase_cpp/parser_fasta.hpp, parser_fastq.hpp). Returns
// false for an empty buffer ("Empty file").
bool fastx_to_stream(const uint8_t* data, size_t len, std::vector<uint8_t>& out);

// Read a whole file, inflating gzip when the name ends in ".gz" (the choice of
// src/seq_source.hpp:196-204). BGZF files (every member sized in its 'BC'
// extra field) are inflated on `threads` host threads, any other gzip file as
// one stream (the reference's GzInput, src/seq_source.hpp:48-141). Returns an
// error message, or "" on success.
std::string read_input_file(const std::string& path, Bytes& out, unsigned threads = 1);

// Page-locked host memory from the CUDA driver (tg_host_alloc); null with a
// message in *err on failure. pinned_free takes only pointers from pinned_alloc (false
// otherwise).
void* pinned_alloc(size_t bytes, std::string* err);
bool pinned_free(void* p);

// The KFF container around n entries (header + variables + raw section start),
// and its closing footer.
std::string kff_header(int k, uint64_t n);
std::string kff_footer();

}  // namespace tgh
