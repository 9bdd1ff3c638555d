// tuna_main.cpp — the `tuna` command line on top of libtuna_gpu.so.
//
// Interface kept identical to the reference CLI (src/CLI.cpp:68-237,
// src/main.cpp:23-95), because scripts depend on it: the flags and their
// limits, `tuna [options] <in...|@list> <out>`, every "tuna: error: ..." text
// with exit code 1, -n rounded up to a power of two, KFF output chosen by -kff
// or a ".kff" output name, the header line and the machine-readable stderr
// lines phase1:/phase2:/superkmers:/n_parts:/unique_kmers:
// (src/pipeline.hpp:174-178). The code is organised differently: one table
// describes every option (name, kind, limit, the field it sets) and a single
// pass over argv consults it; the checks after parsing are a list of
// (condition, message) rules. Both phases run on the GPU; -t sets the host
// threads used to read inputs and format output.
#include <sys/resource.h>

#include <cerrno>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "tuna_gpu.h"

namespace fs = std::filesystem;

namespace {

constexpr uint64_t U16_MAX = 0xFFFFull, U32_MAX = 0xFFFFFFFFull, U64_MAX = ~0ull;

struct Settings {
    std::vector<std::string> inputs;
    std::string output, work_dir;
    uint64_t k = 31, m = 21, parts = 0, threads = 1, ci = 1, cx = U64_MAX, ram_gb = 0;
    bool hide_progress = false, keep_parts = false, phase1_only = false, debug = false, kff = false;
};

// ------------------------------------------------------------------ options
enum class Kind { Number, Text, Switch };

struct Option {
    const char* flag;
    Kind kind;
    uint64_t limit;                       // Number: largest accepted value
    uint64_t Settings::*number;           // Number: destination
    std::string Settings::*text;          // Text: destination
    bool Settings::*on;                   // Switch: destination
    const char* help;
};

const Option OPTIONS[] = {
    {"-k", Kind::Number, U16_MAX, &Settings::k, nullptr, nullptr, "k-mer length (2..63 on the GPU; default 31)"},
    {"-m", Kind::Number, U16_MAX, &Settings::m, nullptr, nullptr, "minimizer length (1..min(k-1, 32); default 21)"},
    {"-n", Kind::Number, U32_MAX, &Settings::parts, nullptr, nullptr,
     "partitions, rounded up to a power of two (default: from the input size)"},
    {"-t", Kind::Number, U32_MAX, &Settings::threads, nullptr, nullptr, "host threads for input and output"},
    {"-ci", Kind::Number, U32_MAX, &Settings::ci, nullptr, nullptr, "drop k-mers seen fewer times (default 1)"},
    {"-cx", Kind::Number, U64_MAX, &Settings::cx, nullptr, nullptr, "drop k-mers seen more times"},
    {"-ram", Kind::Number, U64_MAX >> 30, &Settings::ram_gb, nullptr, nullptr,
     "memory budget in GB (accepted; device memory is budgeted per job)"},
    {"-w", Kind::Text, 0, nullptr, &Settings::work_dir, nullptr, "directory for partition files"},
    {"-hp", Kind::Switch, 0, nullptr, nullptr, &Settings::hide_progress, "no progress lines"},
    {"-kt", Kind::Switch, 0, nullptr, nullptr, &Settings::keep_parts, "keep hash_<p>.superkmers files"},
    {"-tp", Kind::Switch, 0, nullptr, nullptr, &Settings::phase1_only, "stop after phase 1 (partitioning)"},
    {"-dbg", Kind::Switch, 0, nullptr, nullptr, &Settings::debug, "extra device timings on stderr"},
    {"-kff", Kind::Switch, 0, nullptr, nullptr, &Settings::kff, "KFF output (also chosen by a .kff name)"},
};

const Option* find_option(const std::string& flag) {
    for (const Option& o : OPTIONS)
        if (flag == o.flag) return &o;
    return nullptr;
}

void usage(const char* prog) {
    std::ostringstream s;
    s << "tuna (GB300): counts canonical k-mers of FASTA/FASTQ files (plain or .gz)\n\n"
      << "Usage: " << prog << " [options] <input>... <output>\n"
      << "       " << prog << " [options] @<file listing inputs> <output>\n\n";
    for (const Option& o : OPTIONS) {
        std::string lhs = o.flag;
        if (o.kind == Kind::Number) lhs += " <int>";
        if (o.kind == Kind::Text) lhs += " <dir>";
        s << "  " << lhs << std::string(lhs.size() < 12 ? 12 - lhs.size() : 1, ' ') << o.help << "\n";
    }
    s << "  -h, --help  this text\n"
      << "  -v, --version\n\n"
      << "Output is TSV lines <k-mer><TAB><count> unless KFF is asked for.\n";
    std::cerr << s.str();
}

void say_error(const std::string& what) { std::cerr << "tuna: error: " << what << "\n"; }

// Decimal text to an integer as std::stoull reads it (leading blanks and a sign
// allowed, the whole text consumed); false with the reference's message when
// it is not an integer or exceeds `limit`.
bool read_number(const char* flag, const char* text, uint64_t limit, uint64_t& out) {
    errno = 0;
    char* end = nullptr;
    const unsigned long long v = std::strtoull(text, &end, 10);
    const bool converted = end != text && errno != ERANGE;
    if (!converted || *end != '\0') {
        say_error(std::string("invalid integer for ") + flag + ": " + text);
        return false;
    }
    if (v > limit) {
        say_error(std::string("value out of range for ") + flag + ": " + text);
        return false;
    }
    out = v;
    return true;
}

// The inputs named by an @list file, one per non-empty line ("~/" expanded).
bool read_list(std::string path, std::vector<std::string>& out) {
    if (path.rfind("~/", 0) == 0) {
        if (const char* home = std::getenv("HOME")) path = home + path.substr(1);
    }
    std::ifstream in(path);
    if (!in) {
        say_error("cannot open input list: " + path);
        return false;
    }
    for (std::string line; std::getline(in, line);)
        if (!line.empty()) out.push_back(line);
    return true;
}

enum class Parse { Run, Usage, Version };

Parse parse(int argc, char** argv, Settings& s) {
    if (argc < 2) return Parse::Usage;
    std::vector<std::string> loose;
    for (int i = 1; i < argc; ++i) {
        const std::string tok = argv[i];
        if (tok == "-h" || tok == "--help") return Parse::Usage;
        if (tok == "-v" || tok == "--version") return Parse::Version;
        const Option* o = find_option(tok);
        if (!o) {
            if (!tok.empty() && tok[0] == '-') {
                say_error("unknown option: " + tok);
                return Parse::Usage;
            }
            loose.push_back(tok);
            continue;
        }
        if (o->kind == Kind::Switch) {
            s.*(o->on) = true;
            continue;
        }
        if (i + 1 >= argc) {
            say_error(tok + " requires an argument");
            return Parse::Usage;
        }
        const char* val = argv[++i];
        if (o->kind == Kind::Text) s.*(o->text) = val;
        else if (!read_number(o->flag, val, o->limit, s.*(o->number))) return Parse::Usage;
    }
    if (loose.size() < 2) {
        say_error("need at least one input file and an output file");
        return Parse::Usage;
    }
    s.output = loose.back();
    loose.pop_back();
    if (loose.size() == 1 && loose[0][0] == '@') {
        if (!read_list(loose[0].substr(1), s.inputs)) return Parse::Usage;
    } else {
        s.inputs = loose;
    }
    const size_t on = s.output.size();
    if (on >= 4 && s.output.compare(on - 4, 4, ".kff") == 0) s.kff = true;
    // the reference's checks, in its order, with its messages
    const std::string km = "(-k " + std::to_string(s.k) + ")", mm = "(-m " + std::to_string(s.m) + ")";
    const struct {
        bool bad;
        std::string msg;
    } rules[] = {
        {s.inputs.empty(), "no input files"},
        {s.k < 2 || s.k > 256, "k-mer length " + km + " must be in [2, 256]"},
        {s.m < 1 || s.m > 32, "minimizer length " + mm + " must be in [1, 32]"},
        {s.m >= s.k, "minimizer length " + mm + " must be strictly less than k-mer length " + km},
        {s.threads == 0, "number of threads (-t) must be > 0"},
    };
    for (const auto& r : rules)
        if (r.bad) {
            say_error(r.msg);
            return Parse::Usage;
        }
    return Parse::Run;
}

// ------------------------------------------------------------------ partitions
// -n auto: about 2 MB of input per partition (gzip inputs counted at 6x their
// size), a power of two in [16, 4096]. The reference's rule (src/setup.hpp:
// 82-196) also weighs file-descriptor and cache limits; the count only names
// partition files and the n_parts: line, never the counted output.
uint64_t partitions_for(const std::vector<std::string>& files) {
    uint64_t bytes = 0;
    for (const std::string& f : files) {
        std::error_code ec;
        const uint64_t sz = fs::file_size(f, ec);
        if (ec) continue;
        const bool gz = f.size() >= 3 && f.compare(f.size() - 3, 3, ".gz") == 0;
        bytes += gz ? sz * 6 : sz;
    }
    uint64_t n = 16;
    for (const uint64_t want = bytes >> 21; n < want && n < 4096;) n *= 2;
    return n;
}

// -n as the reference's main uses it: the next power of two at or above n
// (1 for 0 and 1), 0 when that power does not fit in 32 bits.
uint64_t as_power_of_two(uint64_t n) {
    if (n > (1ull << 31)) return 0;
    int bits = 0;
    while ((1ull << bits) < n) ++bits;
    return 1ull << bits;
}

// ------------------------------------------------------------------ the run
using Clock = std::chrono::steady_clock;

double since(Clock::time_point t) { return std::chrono::duration<double>(Clock::now() - t).count(); }

int write_partition(uint32_t p, const uint8_t* data, size_t len, void* dir) {
    const std::string path = *static_cast<const std::string*>(dir) + "hash_" + std::to_string(p) + ".superkmers";
    std::ofstream f(path, std::ios::binary);
    if (len) f.write(reinterpret_cast<const char*>(data), (std::streamsize)len);
    return f ? 0 : 1;
}

// One GPU job from the settings; owns the context and the job.
class Session {
public:
    explicit Session(const Settings& s) : s_(s) {}
    ~Session() {
        if (job_) tg_job_end(job_);
        if (ctx_) tg_ctx_destroy(ctx_);
    }

    int run() {
        const Clock::time_point t_all = Clock::now();
        tg_ctx_opts co{};
        co.host_threads = (uint32_t)s_.threads;
        if (tg_ctx_create(&co, &ctx_) != TG_OK) return fail("no usable CUDA device");
        tg_job_opts jo{};
        jo.k = (uint16_t)s_.k;
        jo.m = (uint16_t)s_.m;
        jo.n_parts = (uint32_t)s_.parts;
        jo.ci = s_.ci;
        jo.cx = s_.cx;
        if (tg_job_begin(ctx_, &jo, &job_) != TG_OK) return fail(tg_last_error(ctx_));
        progress("[1/2] partitioning  (GPU, in-memory) ...");
        const Clock::time_point t_p1 = Clock::now();
        for (const std::string& f : s_.inputs)
            if (tg_job_feed_file(job_, f.c_str()) != TG_OK) return fail(tg_last_error(ctx_));
        if (tg_job_run(job_) != TG_OK) return fail(tg_last_error(ctx_));
        tg_job_stats(job_, &st_);
        // the reference's phase 1 covers reading the input and partitioning:
        // the wall time of feeding and running minus the device's phase 2
        const double p2_device = st_.phase2_ms / 1e3;
        const double phase1 = std::max(0.0, since(t_p1) - p2_device);
        if (s_.phase1_only) {
            if (s_.keep_parts && !export_partitions()) return 1;
            std::cerr << "phase1: " << phase1 << "s\n" << "superkmers: " << st_.superkmers << "\n";
            progress("done  (partition only)");
            return 0;
        }
        progress("[2/2] counting  (GPU) ...");
        const Clock::time_point t_out = Clock::now();
        if (tg_job_write(job_, s_.kff ? TG_FMT_KFF : TG_FMT_TSV, s_.output.c_str()) != TG_OK)
            return fail(tg_last_error(ctx_));
        if (s_.keep_parts && !export_partitions()) return 1;
        const double phase2 = p2_device + since(t_out);
        progress("      " + std::to_string(st_.kmers) + " k-mers in  " + std::to_string(st_.out) + " unique out");
        std::cerr << "phase1: " << phase1 << "s\n"
                  << "phase2: " << phase2 << "s\n"
                  << "superkmers: " << st_.superkmers << "\n"
                  << "n_parts: " << s_.parts << "\n"
                  << "unique_kmers: " << st_.out << "\n";
        if (s_.debug)
            std::cerr << "gpu_phase1_s: " << st_.phase1_ms / 1e3 << "\n"
                      << "gpu_phase2_s: " << st_.phase2_ms / 1e3 << "\n"
                      << "h2d_s: " << st_.h2d_ms / 1e3 << "\n"
                      << "gpu_parts: " << st_.gpu_parts << "\n"
                      << "distinct_kmers: " << st_.distinct << "\n";
        if (!s_.hide_progress) {
            char total[32];
            std::snprintf(total, sizeof total, "%.3fs", since(t_all));
            std::cerr << "total: " << total << "\n";
        }
        return 0;
    }

private:
    int fail(const std::string& what) {
        say_error(what);
        return 1;
    }
    void progress(const std::string& line) const {
        if (!s_.hide_progress) std::cerr << line << "\n";
    }
    bool export_partitions() {
        std::string dir = s_.work_dir;
        if (tg_job_export_partitions(job_, write_partition, &dir) == TG_OK) return true;
        fail("cannot write partition files to " + s_.work_dir);
        return false;
    }

    const Settings& s_;
    tg_ctx* ctx_ = nullptr;
    tg_job* job_ = nullptr;
    tg_stats st_{};
};

void raise_open_file_limit() {
    struct rlimit rl{};
    if (getrlimit(RLIMIT_NOFILE, &rl) != 0) return;
    rl.rlim_cur = rl.rlim_max;
    setrlimit(RLIMIT_NOFILE, &rl);
}

}  // namespace

int main(int argc, char* argv[]) {
    Settings s;
    switch (parse(argc, argv, s)) {
        case Parse::Usage:
            usage(argv[0]);
            return 1;
        case Parse::Version:
            std::cerr << "tuna " << tg_version() << "\n";
            return 0;
        case Parse::Run:
            break;
    }
    raise_open_file_limit();
    s.parts = as_power_of_two(s.parts ? s.parts : partitions_for(s.inputs));
    // partition files go to -w, else to tuna_tmp/ beside the output (removed
    // afterwards unless -kt)
    const bool temp_dir = s.work_dir.empty();
    if (temp_dir) {
        fs::path parent = fs::path(s.output).parent_path();
        s.work_dir = ((parent.empty() ? fs::current_path() : parent) / "tuna_tmp").string();
    }
    if (s.work_dir.back() != '/') s.work_dir.push_back('/');
    std::error_code ec;
    fs::create_directories(s.work_dir, ec);
    if (!s.hide_progress) {
        std::ostringstream h;
        h << "tuna  k=" << s.k << "  m=" << s.m << "  n=" << s.parts << "  t=" << s.threads;
        if (s.ci > 1 || s.cx != U64_MAX) h << "  ci=" << s.ci << "  cx=" << s.cx;
        std::cerr << h.str() << "\n";
    }
    int rc = 1;
    try {
        Session job(s);
        rc = job.run();
    } catch (const std::exception& x) {
        say_error(x.what());
    }
    if (!s.keep_parts) {
        if (temp_dir) {
            fs::remove_all(s.work_dir, ec);
        } else {
            for (uint64_t p = 0; p < s.parts; ++p)
                fs::remove(s.work_dir + "hash_" + std::to_string(p) + ".superkmers", ec);
        }
    }
    return rc;
}
