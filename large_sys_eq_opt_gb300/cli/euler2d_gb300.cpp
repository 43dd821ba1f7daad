// euler2d_gb300 -- command-line driver of the GB300 solver with the
// reference driver's interface and outputs (scripts/cpu/main_cpu.cpp):
//
//   euler2d_gb300 [n] [--case shock_bubble|blast_wave] [--solver hll|hllc|exact|force]
//                 [--output | --timing-only | --no-output]
//   extensions:   [--precision fp64|fp32] [--problem blast_256|shock_bubble_1000x396]
//                 [--prefix NAME] [--outdir DIR]
//
// The time loop runs on the device (eu_run): dt, the t_end clip and the
// snapshot schedule never leave the GPU.  Snapshots are copied out when the
// device reaches them and written by a background thread in the exact format
// of write_grid_csv (scripts/cpu/main_cpu.cpp:136-164: header
// i,j,x,y,rho,rhou,rhov,E, interior cells, default stream precision), so the
// CSV writing overlaps the next steps instead of stalling them.
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "euler2d.h"

namespace {

struct Options {
    int n = 1;
    std::string case_name = "shock_bubble";
    std::string solver_name = "hll";
    int solver = EU_HLL;
    bool write_output = false;
    int nsnap = 5;
    eu_precision prec = EU_FP64;
    std::string problem;
    std::string prefix = "gb300";
    std::string outdir = "outputs";
};

// parse_riemann_solver (scripts/cpu/main_cpu.cpp:32-50)
int parse_solver(const std::string& s, std::string& canon) {
    if (s == "hll" || s == "HLL") { canon = "hll"; return EU_HLL; }
    if (s == "hllc" || s == "HLLC") { canon = "hllc"; return EU_HLLC; }
    if (s == "exact" || s == "Exact" || s == "EXACT") { canon = "exact"; return EU_EXACT; }
    if (s == "force" || s == "Force" || s == "FORCE") { canon = "force"; return EU_FORCE; }
    throw std::runtime_error("Unknown Riemann solver: " + s + ". Supported solvers are: hll, hllc, exact, force.");
}

// parse_run_options (scripts/cpu/main_cpu.cpp:67-113) plus the extensions
Options parse(int argc, char** argv) {
    Options o;
    if (argc >= 2 && argv[1][0] != '-') o.n = std::stoi(argv[1]);
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (i == 1 && !a.empty() && a[0] != '-') continue;
        auto next = [&](const char* what) -> std::string {
            if (i + 1 >= argc) throw std::runtime_error(std::string(what) + " requires a value.");
            return argv[++i];
        };
        if (a == "--output") { o.write_output = true; o.nsnap = 5; }
        else if (a == "--timing-only" || a == "--no-output") { o.write_output = false; o.nsnap = 0; }
        else if (a == "--case") o.case_name = next("--case");
        else if (a == "--solver") o.solver = parse_solver(next("--solver"), o.solver_name);
        else if (a == "--precision") {
            const std::string p = next("--precision");
            if (p == "fp64") o.prec = EU_FP64;
            else if (p == "fp32") o.prec = EU_FP32;
            else throw std::runtime_error("--precision must be fp64 or fp32");
        } else if (a == "--problem") o.problem = next("--problem");
        else if (a == "--prefix") o.prefix = next("--prefix");
        else if (a == "--outdir") o.outdir = next("--outdir");
        else throw std::runtime_error("Unknown argument: " + a);
    }
    if (o.n <= 0) throw std::runtime_error("resolution_scale must be positive.");
    return o;
}

struct Snapshot {
    int k;
    double t;
    std::vector<double> aos;
};

// Background CSV writer: snapshots queue here while the device keeps stepping.
class Writer {
public:
    Writer(const eu_case& cfg, std::string stem) : cfg_(cfg), stem_(std::move(stem)), th_([this] { loop(); }) {}
    ~Writer() {
        {
            std::lock_guard<std::mutex> g(m_);
            done_ = true;
        }
        cv_.notify_all();
        th_.join();
    }
    void push(Snapshot s) {
        {
            std::lock_guard<std::mutex> g(m_);
            q_.push_back(std::move(s));
        }
        cv_.notify_all();
    }

private:
    void loop() {
        for (;;) {
            Snapshot s;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return done_ || !q_.empty(); });
                if (q_.empty()) return;
                s = std::move(q_.front());
                q_.pop_front();
            }
            write(s);
        }
    }
    // write_grid_csv (scripts/cpu/main_cpu.cpp:136-164)
    void write(const Snapshot& s) {
        const std::string fn = stem_ + std::to_string(s.k) + ".csv";
        std::ofstream out(fn);
        out << "i,j,x,y,rho,rhou,rhov,E\n";
        const double dx = (cfg_.x_max - cfg_.x_min) / static_cast<double>(cfg_.nx);
        const double dy = (cfg_.y_max - cfg_.y_min) / static_cast<double>(cfg_.ny);
        const int tnx = cfg_.nx + 2 * cfg_.ng;
        for (int j = cfg_.ng; j < cfg_.ng + cfg_.ny; ++j)
            for (int i = cfg_.ng; i < cfg_.ng + cfg_.nx; ++i) {
                const double* U = s.aos.data() + 4 * (static_cast<size_t>(j) * tnx + i);
                const double x = cfg_.x_min + (static_cast<double>(i - cfg_.ng) + 0.5) * dx;
                const double y = cfg_.y_min + (static_cast<double>(j - cfg_.ng) + 0.5) * dy;
                out << i << "," << j << "," << x << "," << y << "," << U[0] << "," << U[1] << "," << U[2] << ","
                    << U[3] << "\n";
            }
        std::cout << "[GB300] Wrote snapshot " << s.k << " at t = " << s.t << " -> " << fn << "\n";
    }

    eu_case cfg_;
    std::string stem_;
    std::mutex m_;
    std::condition_variable cv_;
    std::deque<Snapshot> q_;
    bool done_ = false;
    std::thread th_;
};

int on_snapshot(void* user, int k, long long step, double t, const double* aos, int nx, int ny) {
    (void)step;
    Writer* w = static_cast<Writer*>(user);
    const size_t n = 4 * static_cast<size_t>(nx + 4) * static_cast<size_t>(ny + 4);
    w->push(Snapshot{k, t, std::vector<double>(aos, aos + n)});
    return 0;
}

void die(const std::string& what, const eu_handle* h) {
    throw std::runtime_error(what + ": " + eu_last_error(h));
}

}  // namespace

int main(int argc, char** argv) {
    try {
        const Options opts = parse(argc, argv);
        eu_case cfg{};
        int bc[4] = {EU_BC_TRANSMISSIVE, EU_BC_TRANSMISSIVE, EU_BC_TRANSMISSIVE, EU_BC_TRANSMISSIVE};
        std::string case_label = opts.case_name;
        if (opts.problem.empty()) {
            if (eu_get_case_config(opts.case_name.c_str(), opts.n, &cfg) != EU_OK) die("case", nullptr);
        } else if (opts.problem == "blast_256") {
            cfg = eu_case{256, 256, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25};
            case_label = opts.problem;
        } else if (opts.problem == "shock_bubble_1000x396") {
            cfg = eu_case{1000, 396, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 0.1};
            bc[EU_SIDE_BOTTOM] = bc[EU_SIDE_TOP] = EU_BC_REFLECTIVE;
            case_label = opts.problem;
        } else {
            throw std::runtime_error("Unknown problem: " + opts.problem);
        }
        eu_handle* h = nullptr;
        if (eu_create(&cfg, opts.prec, static_cast<eu_solver>(opts.solver), EU_LIMITER_MINMOD, bc, &h) != EU_OK)
            die("eu_create", nullptr);
        int rc;
        if (opts.problem.empty()) rc = eu_init_reference_case(h, opts.case_name.c_str());
        else if (opts.problem == "blast_256") rc = eu_init_blast(h, 1.0, 1.0, 0.4, 1.0, 1.0, 0.125, 0.1);
        else rc = eu_init_shock_bubble(h, 1.0, 1.0, 1.22, 0.005, 0.035, 0.0445, 0.025, 0.138);
        if (rc != EU_OK) die("initial state", h);

        const int nsnap = opts.write_output ? opts.nsnap : 0;
        std::cout << "[GB300] case_name          : " << case_label << "\n";
        std::cout << "[GB300] riemann_solver     : " << opts.solver_name << "\n";
        std::cout << "[GB300] precision          : " << (opts.prec == EU_FP32 ? "fp32" : "fp64") << "\n";
        std::cout << "[GB300] resolution_scale   : " << opts.n << "\n";
        std::cout << "[GB300] nx                 : " << cfg.nx << "\n";
        std::cout << "[GB300] ny                 : " << cfg.ny << "\n";
        std::cout << "[GB300] total_cells        : " << static_cast<long long>(cfg.nx) * cfg.ny << "\n";
        std::cout << "[GB300] write_output       : " << (opts.write_output ? "true" : "false") << "\n";
        std::cout << "[GB300] num_snapshots      : " << nsnap << "\n";

        eu_run_info info{};
        const auto t0 = std::chrono::steady_clock::now();
        {
            std::string stem;
            if (opts.write_output) {
                std::filesystem::create_directories(opts.outdir);
                std::ostringstream ss;
                ss << opts.outdir << "/" << opts.prefix << "_" << case_label << "_" << opts.solver_name << "_n"
                   << opts.n << "_snapshot_";
                stem = ss.str();
            }
            Writer writer(cfg, stem);
            rc = eu_run(h, cfg.t_end, nsnap, nsnap ? on_snapshot : nullptr, &writer, &info);
        }
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (rc != EU_OK) die("eu_run", h);
        std::cout << "[GB300] Finished.\n";
        std::cout << "[GB300] Final time = " << info.t << "\n";
        std::cout << "[GB300] Total steps = " << info.steps << "\n";
        std::cout << "[GB300] Wall seconds = " << secs << "\n";
        if (!opts.write_output) std::cout << "[GB300] Output disabled. No files were written.\n";
        eu_destroy(h);
        return 0;
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
}
