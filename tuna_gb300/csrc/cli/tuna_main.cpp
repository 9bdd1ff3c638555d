// tuna_main.cpp — the `tuna` command line on top of libtuna_gpu.so.
//
// Same flags, messages and exit codes as the reference CLI (src/CLI.cpp:68-237,
// src/main.cpp:23-95): `tuna [options] <in...|@list> <out>`, errors as
// "tuna: error: ..." with exit code 1, KFF output chosen by -kff or a .kff
// extension, the machine-readable stderr lines phase1:/phase2:/superkmers:/
// n_parts:/unique_kmers: (src/pipeline.hpp:174-178). Both phases run on the GPU;
// -t sets the host threads used to read inputs and format output.
#include <sys/resource.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <limits>
#include <string>
#include <vector>

#include "tuna_gpu.h"

namespace fs = std::filesystem;

struct Config {
    std::vector<std::string> input_files;
    std::string output_file, work_dir;
    uint16_t k = 31, l = 21;
    uint32_t num_partitions = 0, num_threads = 1;
    uint32_t ci = 1;
    uint64_t cx = std::numeric_limits<uint64_t>::max();
    bool hide_progress = false, keep_tmp = false, partition_only = false, debug_stats = false,
         output_kff = false;
    uint64_t ram_budget_bytes = 0;
};

static void print_usage(const char* prog) {
    std::cerr << "tuna — streaming k-mer counter (GB300)\n\n"
                 "Usage:\n"
                 "  " << prog << " [options] <input1.fa [input2.fa ...]> <output_file>\n"
                 "  " << prog << " [options] @<input_list_file>          <output_file>\n\n"
                 "Options:\n"
                 "  -k  <int>   k-mer length               [default: 31] (GPU path: 2..63)\n"
                 "  -m  <int>   minimizer length            [default: 21] (1..min(k-1, 32))\n"
                 "  -n  <int>   number of partitions        [default: auto, ~2 MB input/partition]\n"
                 "  -t  <int>   host threads                [default: 1]\n"
                 "  -ci <int>   minimum k-mer count         [default: 1]\n"
                 "  -cx <int>   maximum k-mer count         [default: max]\n"
                 "  -ram <int>  RAM budget in GB            [accepted; phase 2 budgets device memory\n"
                 "              and runs in passes when a job does not fit]\n"
                 "  -w  <dir>   working directory for temp files\n"
                 "              [default: tuna_tmp/ next to output file]\n\n"
                 "  -hp         hide progress messages\n"
                 "  -kt         keep partition files (hash_<p>.superkmers) in the work dir\n"
                 "  -tp         stop after partitioning (phase 1 only)\n"
                 "  -dbg        debug stats\n"
                 "  -kff        write output in KFF binary format (auto-detected from .kff extension)\n"
                 "  -h/--help   show this help\n"
                 "  -v/--version print version\n\n"
                 "Output: plain text TSV (<kmer>\\t<count>) by default; use -kff for KFF binary.\n";
}

static bool parse_args(int argc, char* argv[], Config& cfg) {
    if (argc < 2) return false;
    std::vector<std::string> positionals;
    for (int i = 1; i < argc; ++i) {
        const std::string arg = argv[i];
        if (arg == "-h" || arg == "--help") return false;
        if (arg == "-v" || arg == "--version") {
            std::cerr << "tuna " << tg_version() << "\n";
            std::exit(0);
        }
        auto next_val = [&](const char* flag) -> const char* {
            if (i + 1 >= argc) {
                std::cerr << "tuna: error: " << flag << " requires an argument\n";
                return nullptr;
            }
            return argv[++i];
        };
        auto parse_u64 = [&](const char* flag, const char* txt, uint64_t max, uint64_t& out) -> bool {
            try {
                const std::string s(txt);
                size_t pos = 0;
                const unsigned long long v = std::stoull(s, &pos, 10);
                if (pos != s.size()) {
                    std::cerr << "tuna: error: invalid integer for " << flag << ": " << s << "\n";
                    return false;
                }
                if (v > max) {
                    std::cerr << "tuna: error: value out of range for " << flag << ": " << s << "\n";
                    return false;
                }
                out = v;
                return true;
            } catch (const std::exception&) {
                std::cerr << "tuna: error: invalid integer for " << flag << ": " << txt << "\n";
                return false;
            }
        };
        uint64_t v = 0;
        const char* t = nullptr;
        if (arg == "-k") {
            if (!(t = next_val("-k")) || !parse_u64("-k", t, 65535, v)) return false;
            cfg.k = (uint16_t)v;
        } else if (arg == "-m") {
            if (!(t = next_val("-m")) || !parse_u64("-m", t, 65535, v)) return false;
            cfg.l = (uint16_t)v;
        } else if (arg == "-n") {
            if (!(t = next_val("-n")) || !parse_u64("-n", t, 0xFFFFFFFFull, v)) return false;
            cfg.num_partitions = (uint32_t)v;
        } else if (arg == "-ci") {
            if (!(t = next_val("-ci")) || !parse_u64("-ci", t, 0xFFFFFFFFull, v)) return false;
            cfg.ci = (uint32_t)v;
        } else if (arg == "-cx") {
            if (!(t = next_val("-cx")) || !parse_u64("-cx", t, std::numeric_limits<uint64_t>::max(), v)) return false;
            cfg.cx = v;
        } else if (arg == "-t") {
            if (!(t = next_val("-t")) || !parse_u64("-t", t, 0xFFFFFFFFull, v)) return false;
            cfg.num_threads = (uint32_t)v;
        } else if (arg == "-ram") {
            if (!(t = next_val("-ram")) || !parse_u64("-ram", t, std::numeric_limits<uint64_t>::max() >> 30, v))
                return false;
            cfg.ram_budget_bytes = v << 30;
        } else if (arg == "-w") {
            if (!(t = next_val("-w"))) return false;
            cfg.work_dir = t;
        } else if (arg == "-dbg") {
            cfg.debug_stats = true;
        } else if (arg == "-kff") {
            cfg.output_kff = true;
        } else if (arg == "-hp") {
            cfg.hide_progress = true;
        } else if (arg == "-kt") {
            cfg.keep_tmp = true;
        } else if (arg == "-tp") {
            cfg.partition_only = true;
        } else if (!arg.empty() && arg[0] == '-') {
            std::cerr << "tuna: error: unknown option: " << arg << "\n";
            return false;
        } else {
            positionals.push_back(arg);
        }
    }
    if (positionals.size() < 2) {
        std::cerr << "tuna: error: need at least one input file and an output file\n";
        return false;
    }
    cfg.output_file = positionals.back();
    positionals.pop_back();
    if (positionals.size() == 1 && positionals[0][0] == '@') {
        std::string list_path = positionals[0].substr(1);
        if (list_path.size() >= 2 && list_path[0] == '~' && list_path[1] == '/') {
            const char* home = std::getenv("HOME");
            if (home) list_path = std::string(home) + list_path.substr(1);
        }
        std::ifstream list_f(list_path);
        if (!list_f) {
            std::cerr << "tuna: error: cannot open input list: " << list_path << "\n";
            return false;
        }
        std::string line;
        while (std::getline(list_f, line))
            if (!line.empty()) cfg.input_files.push_back(line);
    } else {
        cfg.input_files = std::move(positionals);
    }
    if (cfg.input_files.empty()) {
        std::cerr << "tuna: error: no input files\n";
        return false;
    }
    if (!cfg.output_kff) {
        const auto& of = cfg.output_file;
        if (of.size() >= 4 && of.compare(of.size() - 4, 4, ".kff") == 0) cfg.output_kff = true;
    }
    if (cfg.k < 2 || cfg.k > 256) {
        std::cerr << "tuna: error: k-mer length (-k " << cfg.k << ") must be in [2, 256]\n";
        return false;
    }
    if (cfg.l < 1 || cfg.l > 32) {
        std::cerr << "tuna: error: minimizer length (-m " << cfg.l << ") must be in [1, 32]\n";
        return false;
    }
    if (cfg.l >= cfg.k) {
        std::cerr << "tuna: error: minimizer length (-m " << cfg.l
                  << ") must be strictly less than k-mer length (-k " << cfg.k << ")\n";
        return false;
    }
    if (cfg.num_threads == 0) {
        std::cerr << "tuna: error: number of threads (-t) must be > 0\n";
        return false;
    }
    return true;
}

// Partition count for -n auto: the reference sizes partitions for ~2 MB of input
// each (setup.hpp:82-196), rounded to a power of two in [16, 4096]; the count
// only names exported partition files and the n_parts: line, never the output.
static uint32_t auto_partitions(const std::vector<std::string>& files) {
    uint64_t total = 0;
    for (const auto& f : files) {
        std::error_code ec;
        uint64_t sz = fs::file_size(f, ec);
        if (ec) continue;
        if (f.size() >= 3 && f.compare(f.size() - 3, 3, ".gz") == 0) sz *= 6;
        total += sz;
    }
    uint64_t n = 16;
    while (n < (total >> 21) && n < 4096) n <<= 1;
    return (uint32_t)n;
}

// -n rounded up to a power of two (the reference's -n semantics, main.cpp:52):
// the smallest 2^j >= n, 1 for n <= 1, and 0 where 2^j would not fit in 32 bits.
static uint32_t round_pow2(uint32_t n) {
    if (n > (1u << 31)) return 0;
    uint32_t p = 1;
    while (p < n) p <<= 1;
    return p;
}

static double secs(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

struct PartWriter {
    std::string dir;
    bool ok = true;
};
static int part_sink(uint32_t p, const uint8_t* data, size_t len, void* u) {
    PartWriter* w = static_cast<PartWriter*>(u);
    std::ofstream f(w->dir + "hash_" + std::to_string(p) + ".superkmers", std::ios::binary);
    if (len) f.write(reinterpret_cast<const char*>(data), (std::streamsize)len);
    if (!f) { w->ok = false; return 1; }
    return 0;
}

static int run(const Config& cfg) {
    const auto t_start = std::chrono::steady_clock::now();
    tg_ctx_opts co{};
    co.device = 0;
    co.host_threads = cfg.num_threads;
    tg_ctx* ctx = nullptr;
    if (tg_ctx_create(&co, &ctx) != TG_OK) {
        std::cerr << "tuna: error: no usable CUDA device\n";
        return 1;
    }
    tg_job_opts jo{};
    jo.k = cfg.k;
    jo.m = cfg.l;
    jo.n_parts = cfg.num_partitions;
    jo.ci = cfg.ci;
    jo.cx = cfg.cx;
    tg_job* job = nullptr;
    auto fail = [&](const std::string& what) {
        std::cerr << "tuna: error: " << what << "\n";
        if (job) tg_job_end(job);
        tg_ctx_destroy(ctx);
        return 1;
    };
    if (tg_job_begin(ctx, &jo, &job) != TG_OK) return fail(tg_last_error(ctx));
    if (!cfg.hide_progress) std::cerr << "[1/2] partitioning  (GPU, in-memory) ...\n";
    const auto t_part = std::chrono::steady_clock::now();
    for (const auto& f : cfg.input_files)
        if (tg_job_feed_file(job, f.c_str()) != TG_OK) return fail(tg_last_error(ctx));
    if (tg_job_run(job) != TG_OK) return fail(tg_last_error(ctx));
    tg_stats st{};
    tg_job_stats(job, &st);
    // phase boundaries as the reference prints them: phase 1 = input + partitioning
    const double total_run = secs(t_part);
    const double dev_p2 = st.phase2_ms / 1000.0;
    const double t_phase1 = std::max(0.0, total_run - dev_p2);
    if (cfg.partition_only) {
        if (cfg.keep_tmp) {
            PartWriter pw{cfg.work_dir};
            if (tg_job_export_partitions(job, part_sink, &pw) != TG_OK || !pw.ok)
                return fail("cannot write partition files to " + cfg.work_dir);
        }
        std::cerr << "phase1: " << t_phase1 << "s\n"
                  << "superkmers: " << st.superkmers << "\n";
        if (!cfg.hide_progress) std::cerr << "done  (partition only)\n";
        tg_job_end(job);
        tg_ctx_destroy(ctx);
        return 0;
    }
    if (!cfg.hide_progress) std::cerr << "[2/2] counting  (GPU) ...\n";
    const auto t2 = std::chrono::steady_clock::now();
    if (tg_job_write(job, cfg.output_kff ? TG_FMT_KFF : TG_FMT_TSV, cfg.output_file.c_str()) != TG_OK)
        return fail(tg_last_error(ctx));
    if (cfg.keep_tmp) {
        PartWriter pw{cfg.work_dir};
        if (tg_job_export_partitions(job, part_sink, &pw) != TG_OK || !pw.ok)
            return fail("cannot write partition files to " + cfg.work_dir);
    }
    const double t_phase2 = dev_p2 + secs(t2);
    if (!cfg.hide_progress)
        std::cerr << "      " << st.kmers << " k-mers in  " << st.out << " unique out\n";
    std::cerr << "phase1: " << t_phase1 << "s\n"
              << "phase2: " << t_phase2 << "s\n"
              << "superkmers: " << st.superkmers << "\n"
              << "n_parts: " << cfg.num_partitions << "\n"
              << "unique_kmers: " << st.out << "\n";
    if (cfg.debug_stats)
        std::cerr << "gpu_phase1_s: " << st.phase1_ms / 1000.0 << "\n"
                  << "gpu_phase2_s: " << st.phase2_ms / 1000.0 << "\n"
                  << "h2d_s: " << st.h2d_ms / 1000.0 << "\n"
                  << "gpu_parts: " << st.gpu_parts << "\n"
                  << "distinct_kmers: " << st.distinct << "\n";
    if (!cfg.hide_progress) {
        char buf[32];
        std::snprintf(buf, sizeof buf, "%.3fs", secs(t_start));
        std::cerr << "total: " << buf << "\n";
    }
    tg_job_end(job);
    tg_ctx_destroy(ctx);
    return 0;
}

int main(int argc, char* argv[]) {
    Config cfg;
    if (!parse_args(argc, argv, cfg)) {
        print_usage(argv[0]);
        return 1;
    }
    {
        struct rlimit rl{};
        if (getrlimit(RLIMIT_NOFILE, &rl) == 0) {
            rl.rlim_cur = rl.rlim_max;
            setrlimit(RLIMIT_NOFILE, &rl);
        }
    }
    if (cfg.num_partitions == 0) cfg.num_partitions = auto_partitions(cfg.input_files);
    cfg.num_partitions = round_pow2(cfg.num_partitions);
    bool own_work_dir = false;
    if (cfg.work_dir.empty()) {
        fs::path out_parent = fs::path(cfg.output_file).parent_path();
        if (out_parent.empty()) out_parent = fs::current_path();
        cfg.work_dir = (out_parent / "tuna_tmp").string();
        own_work_dir = true;
    }
    if (cfg.work_dir.back() != '/') cfg.work_dir += '/';
    std::error_code ec;
    fs::create_directories(cfg.work_dir, ec);
    if (!cfg.hide_progress) {
        std::cerr << "tuna  k=" << cfg.k << "  m=" << cfg.l << "  n=" << cfg.num_partitions
                  << "  t=" << cfg.num_threads;
        if (cfg.ci > 1 || cfg.cx != std::numeric_limits<uint64_t>::max())
            std::cerr << "  ci=" << cfg.ci << "  cx=" << cfg.cx;
        std::cerr << "\n";
    }
    int rc = 1;
    try {
        rc = run(cfg);
    } catch (const std::exception& e) {
        std::cerr << "tuna: error: " << e.what() << "\n";
        rc = 1;
    }
    if (!cfg.keep_tmp) {
        if (own_work_dir) fs::remove_all(cfg.work_dir, ec);
        else
            for (size_t p = 0; p < cfg.num_partitions; ++p)
                fs::remove(cfg.work_dir + "hash_" + std::to_string(p) + ".superkmers", ec);
    }
    return rc;
}
