// posi_cli.cpp -- the `posidonius` command (src/main.rs), over the C ABI.
//
//   posidonius start <case.json> <recovery_snapshot.bin|.json> <history.bin> [-l seconds] [-s]
//   posidonius resume <recovery_snapshot.bin|.json> <history.bin> [-l seconds] [-s]
//              [--historic-snapshot-period days] [--recovery-snapshot-period days] [--time-limit days]
//
// A snapshot path ending in ".json" is JSON, any other bincode, as in the
// reference (src/integrator/output.rs:43-51, 186-191).  Both take
// `--mode exact|fast` (default exact: results bit-identical to the
// reference; fast: contracted arithmetic, see posi_mode) and `--device k`.
// Messages, the refusal to overwrite files on start, the history truncation
// on resume and the snapshot schedule follow src/main.rs:10-202: without an
// execution limit a recovery snapshot is written at every recovery trigger;
// with one, only when the limit is reached.  Fatal conditions print a PANIC
// line and exit with status 101, as a Rust panic does.
#include <chrono>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>

#include <cuda_runtime.h>

#include "../../include/posidonius_gb300.h"

namespace {

std::string utc_stamp() {
    std::time_t now = std::time(nullptr);
    std::tm g;
    gmtime_r(&now, &g);
    char buf[32];
    std::strftime(buf, sizeof buf, "%Y.%m.%d %H:%M:%S", &g);
    return buf;
}

void say(const char* level, const char* fmt, ...) {
    std::printf("[%s %s UTC] ", level, utc_stamp().c_str());
    va_list ap;
    va_start(ap, fmt);
    std::vprintf(fmt, ap);
    va_end(ap);
    std::printf("\n");
    std::fflush(stdout);
}

[[noreturn]] void panic(const char* fmt, ...) {
    std::printf("[PANIC %s UTC] ", utc_stamp().c_str());
    va_list ap;
    va_start(ap, fmt);
    std::vprintf(fmt, ap);
    va_end(ap);
    std::printf("\n");
    std::fflush(stdout);
    std::exit(101);
}

bool exists(const std::string& p) {
    std::FILE* f = std::fopen(p.c_str(), "rb");
    if (!f) return false;
    std::fclose(f);
    return true;
}

int usage() {
    std::fprintf(stderr,
                 "usage:\n"
                 "  posidonius start <start_case_filename> <snapshot_filename> <historic_snapshot_filename>\n"
                 "                   [-l|--limit seconds] [-s|--silent] [--mode exact|fast] [--device k]\n"
                 "  posidonius resume <resume_case_filename> <historic_snapshot_filename>\n"
                 "                   [-l|--limit seconds] [-s|--silent] [--historic-snapshot-period days]\n"
                 "                   [--recovery-snapshot-period days] [--time-limit days] [--mode exact|fast]\n"
                 "                   [--device k]\n");
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
    const auto timer = std::chrono::steady_clock::now();
    if (argc < 2) return usage();
    const std::string cmd = argv[1];
    const bool resume = cmd == "resume";
    if (!resume && cmd != "start") return usage();
    std::string positional[3];
    int npos = 0;
    uint64_t limit_s = 0;
    bool silent = false;
    double new_hist = -1., new_rec = -1., new_tl = -1.;
    int mode = POSI_MODE_EXACT, device = 0;
    for (int i = 2; i < argc; ++i) {
        const std::string a = argv[i];
        auto value = [&]() -> const char* {
            if (i + 1 >= argc) { std::fprintf(stderr, "missing value for %s\n", a.c_str()); std::exit(2); }
            return argv[++i];
        };
        if (a == "-l" || a == "--limit") {
            limit_s = std::strtoull(value(), nullptr, 10);
        } else if (a == "-s" || a == "--silent") {
            silent = true;
        } else if (a == "--mode") {
            const std::string m = value();
            if (m == "exact") mode = POSI_MODE_EXACT;
            else if (m == "fast") mode = POSI_MODE_FAST;
            else return usage();
        } else if (a == "--device") {
            device = std::atoi(value());
        } else if (resume && a == "--historic-snapshot-period") {
            new_hist = std::strtod(value(), nullptr);
        } else if (resume && a == "--recovery-snapshot-period") {
            new_rec = std::strtod(value(), nullptr);
        } else if (resume && a == "--time-limit") {
            new_tl = (double)std::strtoull(value(), nullptr, 10);
        } else if (!a.empty() && a[0] == '-') {
            return usage();
        } else {
            if (npos >= (resume ? 2 : 3)) return usage();
            positional[npos++] = a;
        }
    }
    if (npos != (resume ? 2 : 3)) return usage();
    const std::string first = positional[0];
    const std::string snapshot = resume ? positional[0] : positional[1];
    const std::string history = resume ? positional[1] : positional[2];

    if (cudaSetDevice(device) != cudaSuccess) panic("cannot select CUDA device %d", device);

    // src/integrator/output.rs:178-203 restore_snapshot
    int st = 0;
    posi_handle* h = exists(first) ? posi_universe_from_json(first.c_str(), mode, &st) : nullptr;
    if (!h) {
        panic("It was not possible to %s the simulation (%s)", resume ? "resume" : "start",
              exists(first) ? posi_last_error() : "File does not exist");
    }
    double t = 0.;
    posi_get_current_time(h, &t);
    if (t == 0.) {
        say("INFO", "Created new simulation based on '%s'.", first.c_str());
        if (posi_initialize_physical_values(h) != POSI_OK) panic("%s", posi_last_error());
    } else {
        say("INFO", "Restored previous simulation from '%s'.", first.c_str());
        const double years = t / 365.25;
        say("INFO", "Continuing from year %.0f (%.1e).", years, years);
    }
    if (posi_set_snapshot_periods(h, new_hist, new_rec) != POSI_OK) panic("%s", posi_last_error());
    if (posi_set_time_limit(h, new_tl) != POSI_OK) panic("%s", posi_last_error());

    int64_t n_hist = 0, n = 0;
    posi_get_n_historic_snapshots(h, &n_hist);
    posi_get_n_particles(h, &n);
    const int64_t expected = n_hist * 156 * n;
    if (!resume && exists(snapshot)) panic("File '%s' already exists.", snapshot.c_str());
    if (!resume && exists(history)) panic("File '%s' already exists.", history.c_str());
    if (posi_open_history(h, history.c_str(), expected) != POSI_OK) panic("%s", posi_last_error());

    // src/main.rs:158-176
    const auto started = std::chrono::steady_clock::now();
    const bool limited = limit_s != 0;
    // with an execution limit the elapsed time is checked every `chunk` steps
    const int64_t chunk = limited ? 256 : (int64_t)1 << 40;
    for (;;) {
        int64_t done = 0;
        int rec = 0;
        const int rc = posi_iterate(h, chunk, &done, &rec);
        if (rc == POSI_COMPLETED) {
            say("INFO", "Simulation completed '%s'.", first.c_str());
            break;
        }
        if (rc == POSI_ERR_PHYSICS) panic("%s", posi_last_error());
        if (rc != POSI_OK) {
            say("INFO", "%s '%s'.", posi_last_error(), first.c_str());
            break;
        }
        if (!silent) {
            // src/integrator/whfast.rs:256-260 progress line
            double now = 0., dt = 0.;
            posi_get_current_time(h, &now);
            int64_t si[POSI_SI_COUNT];
            double sf[POSI_SF_COUNT];
            if (posi_get_state(h, si, sf, nullptr, nullptr, nullptr) == POSI_OK) dt = sf[POSI_SF_DT];
            const double years = now / 365.25;
            std::printf("Year: %.0f (%.1e) | Time step: %.3f days                    \r", years, years, dt);
            std::fflush(stdout);
        }
        if (limited) {
            const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - started).count();
            if (elapsed >= (double)limit_s) {
                if (posi_write_recovery_snapshot(h, snapshot.c_str()) != POSI_OK) panic("%s", posi_last_error());
                say("WARNING", "Reached execution time limit before simulation completion");
                break;
            }
        } else if (rec) {
            if (posi_write_recovery_snapshot(h, snapshot.c_str()) != POSI_OK) panic("%s", posi_last_error());
        }
    }
    posi_close_history(h);
    posi_destroy(h);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - timer).count();
    if (!resume) say("INFO", "Execution time: %g seconds", secs);
    else say("INFO", "Execution time since last resume: %g seconds", secs);
    return 0;
}
