// run_campaign_gpu — the reference's campaign runner (apps/run_campaign.cpp) on the GPU path.
//
// Same command line (run_campaign.cpp:47-76, :185-285) and the same raw CSV schema
// (instrument/csv.hpp:11-137: one row per method x start x seed x repetition, header written
// when the file is empty), so the reference's analysis scripts read its output unchanged.
// Each solve runs through the native GPU drivers of numa/gpu/numa_gpu.hpp; t_F, t_JVP, t_D2 and
// t_prec are CUDA-event times of the primitives, t_total the host wall time of the solve.
//
// Problems: bratu (Bratu3D with mg / jacobi / none).  Starts: natural, perturbed (the
// reference's seeded Gaussian perturbation of a start file, run_campaign.cpp:304-328),
// continuation, coarse.  Extensions: --device, --mg-precision fp64|fp32, --jvp analytic|fd.
//
//   run_campaign_gpu --phase calibration --problem bratu --n 31 --param 6.93 --precond jacobi \
//       --methods nk,cheb,rec --start natural --warmup 1 --reps 7 --out calib.csv --commit SHA
#include "numa/gpu/numa_gpu.hpp"

#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <sys/resource.h>
#include <vector>

namespace {

using numa::gpu::DVec;

struct Args {
    std::string phase = "exploratory", problem = "bratu", family = "B1", precond = "mg";
    std::string methods = "nk,cheb,rec", start = "natural", start_file, start_id;
    std::string dist = "near,mid,far", out = "campaign.csv", commit;
    std::size_t n = 31;
    double param = 1.0;
    double rtol = 1e-8;
    std::size_t max_nl = 50;
    double eta_init = 0.5, eta_max = 0.9, gamma = 0.9, alpha = 2.0, eta2_factor = 10.0, eta2_max = 0.5;
    unsigned seeds = 12;
    int warmup = 1, reps = 7;
    std::size_t restart = 50, maxlin = 500;
    int device = 0;
    int mg_precision = NUMA_GPU_FP64;
    int jvp_mode = NUMA_GPU_DERIV_ANALYTIC;
};

bool to_size(const char* t, std::size_t& v) {
    if (!t || !*t || *t == '-') return false;
    errno = 0;
    char* e = nullptr;
    const unsigned long long r = std::strtoull(t, &e, 10);
    if (errno || e == t || *e || r == 0) return false;
    v = static_cast<std::size_t>(r);
    return true;
}
bool to_int(const char* t, int& v, int lo) {
    if (!t || !*t) return false;
    errno = 0;
    char* e = nullptr;
    const long r = std::strtol(t, &e, 10);
    if (errno || e == t || *e || r < lo || r > std::numeric_limits<int>::max()) return false;
    v = static_cast<int>(r);
    return true;
}
bool to_double(const char* t, double& v) {
    if (!t || !*t) return false;
    errno = 0;
    char* e = nullptr;
    const double r = std::strtod(t, &e);
    if (errno || e == t || *e || !std::isfinite(r)) return false;
    v = r;
    return true;
}

std::vector<std::string> split(const std::string& s) {
    std::vector<std::string> out;
    std::stringstream ss(s);
    std::string tok;
    while (std::getline(ss, tok, ','))
        if (!tok.empty()) out.push_back(tok);
    return out;
}

double rho_for(const std::string& d) {
    if (d == "near") return 0.05;
    if (d == "mid") return 0.20;
    if (d == "far") return 0.50;
    return -1.0;
}

bool parse(int argc, char** argv, Args& a) {
    if ((argc - 1) % 2 != 0) return false;
    if (const char* env = std::getenv("NUMA_COMMIT"); env && *env) a.commit = env;
    for (int i = 1; i < argc; i += 2) {
        const std::string k = argv[i];
        const char* v = argv[i + 1];
        unsigned u = 0;
        if (k == "--phase") a.phase = v;
        else if (k == "--problem") a.problem = v;
        else if (k == "--family") a.family = v;
        else if (k == "--precond") a.precond = v;
        else if (k == "--methods") a.methods = v;
        else if (k == "--start") a.start = v;
        else if (k == "--start-file") a.start_file = v;
        else if (k == "--start-id") a.start_id = v;
        else if (k == "--dist") a.dist = v;
        else if (k == "--out") a.out = v;
        else if (k == "--commit") a.commit = v;
        else if (k == "--n") { if (!to_size(v, a.n)) return false; }
        else if (k == "--param") { if (!to_double(v, a.param)) return false; }
        else if (k == "--rtol") { if (!to_double(v, a.rtol)) return false; }
        else if (k == "--max-nl") { if (!to_size(v, a.max_nl)) return false; }
        else if (k == "--eta-init") { if (!to_double(v, a.eta_init)) return false; }
        else if (k == "--eta-max") { if (!to_double(v, a.eta_max)) return false; }
        else if (k == "--gamma") { if (!to_double(v, a.gamma)) return false; }
        else if (k == "--alpha") { if (!to_double(v, a.alpha)) return false; }
        else if (k == "--eta2-factor") { if (!to_double(v, a.eta2_factor)) return false; }
        else if (k == "--eta2-max") { if (!to_double(v, a.eta2_max)) return false; }
        else if (k == "--seeds") {
            std::size_t s = 0;
            if (!to_size(v, s) || s > std::numeric_limits<unsigned>::max()) return false;
            u = static_cast<unsigned>(s);
            a.seeds = u;
        }
        else if (k == "--warmup") { if (!to_int(v, a.warmup, 0)) return false; }
        else if (k == "--reps") { if (!to_int(v, a.reps, 1)) return false; }
        else if (k == "--restart") { if (!to_size(v, a.restart)) return false; }
        else if (k == "--maxlin") { if (!to_size(v, a.maxlin)) return false; }
        else if (k == "--device") { if (!to_int(v, a.device, 0)) return false; }
        else if (k == "--mg-precision") {
            if (std::string(v) == "fp64") a.mg_precision = NUMA_GPU_FP64;
            else if (std::string(v) == "fp32") a.mg_precision = NUMA_GPU_FP32;
            else return false;
        } else if (k == "--jvp") {
            if (std::string(v) == "analytic") a.jvp_mode = NUMA_GPU_DERIV_ANALYTIC;
            else if (std::string(v) == "fd") a.jvp_mode = NUMA_GPU_DERIV_FD;
            else return false;
        } else return false;
    }
    const bool phase_ok = a.phase == "exploratory" || a.phase == "calibration" || a.phase == "confirmation";
    const bool start_ok = a.start == "natural" || a.start == "perturbed" || a.start == "continuation" ||
                          a.start == "coarse";
    if (!phase_ok || !start_ok || a.out.empty() || a.commit.empty() || !(a.rtol > 0.0) || a.max_nl == 0 ||
        !(a.eta_init > 0.0) || !(a.eta_init <= a.eta_max) || !(a.eta_max > 0.0 && a.eta_max < 1.0) ||
        !(a.gamma > 0.0) || !(a.alpha > 0.0) || !(a.eta2_factor > 0.0) || !(a.eta2_max > 0.0 && a.eta2_max < 1.0) ||
        a.restart == 0 || a.maxlin == 0)
        return false;
    if (a.problem != "bratu") return false;  // the other problem families are not on this path
    if (a.precond != "mg" && a.precond != "jacobi" && a.precond != "none") return false;
    const auto ms = split(a.methods);
    if (ms.empty()) return false;
    for (const auto& m : ms)
        if (m != "nk" && m != "cheb" && m != "rec" && m != "tf2018") return false;
    if (a.start == "perturbed") {
        if (a.start_file.empty() || a.start_id.empty() || a.seeds == 0) return false;
        for (const auto& d : split(a.dist))
            if (rho_for(d) <= 0.0) return false;
    } else if ((a.start == "continuation" || a.start == "coarse") && (a.start_file.empty() || a.start_id.empty())) {
        return false;
    }
    return true;
}

bool load_vector(const std::string& path, std::size_t expected, DVec& values) {
    std::ifstream in(path);
    if (!in) return false;
    values.clear();
    double v = 0.0;
    while (in >> v) {
        if (!std::isfinite(v)) return false;
        values.push_back(v);
    }
    return in.eof() && values.size() == expected;
}

double l2(const DVec& a) {
    double s = 0.0;
    for (double v : a) s += v * v;
    return std::sqrt(s);
}

// The reference's controlled perturbation: a Gaussian direction from mt19937_64 seeded with
// seed * 7919 + 13, scaled to rho * ||reference|| (run_campaign.cpp:304-328).
DVec perturb(const DVec& ref, double rho, unsigned seed) {
    std::mt19937_64 gen(static_cast<unsigned long long>(seed) * 7919ULL + 13ULL);
    std::normal_distribution<double> normal(0.0, 1.0);
    DVec dir(ref.size());
    for (double& v : dir) v = normal(gen);
    const double dn = l2(dir), rn = l2(ref);
    if (!(dn > 0.0) || !(rn > 0.0)) return {};
    const double scale = rho * rn / dn;
    DVec out = ref;
    for (std::size_t i = 0; i < out.size(); ++i) out[i] += scale * dir[i];
    return out;
}

long max_rss_kb() {
    struct rusage u {};
    if (getrusage(RUSAGE_SELF, &u) != 0) return -1;
    return u.ru_maxrss;
}

const char* kHeader =
    "phase,problem,family,n,N,param,instance_id,method,precond,start_kind,start_id,"
    "distance,rho_x,seed,success,nonlinear_iters,n_F,n_JVP,n_D2,n_lin,"
    "n_lin_failures,n_prec,"
    "t_setup,t_F,t_JVP,t_D2,t_prec,t_total,max_rss_kb,residual_rel,"
    "threads,repetition,rtol,max_nl,eta_init,eta_max,gamma,alpha,"
    "eta2_factor,eta2_max,restart,maxlin,commit";

bool append_row(const Args& a, std::size_t N, const std::string& method, const std::string& start_id,
                const std::string& distance, double rho, unsigned seed, const numa::gpu::KrylovResult& r,
                double t_setup, double t_total, int repetition) {
    bool header = true;
    if (FILE* f = std::fopen(a.out.c_str(), "r")) {
        std::fseek(f, 0, SEEK_END);
        header = std::ftell(f) == 0;
        std::fclose(f);
    }
    FILE* f = std::fopen(a.out.c_str(), "a");
    if (!f) return false;
    if (header) std::fprintf(f, "%s\n", kHeader);
    const std::string instance = "lambda=" + std::to_string(a.param);
    const double rel = r.res0 > 0.0 ? r.res / r.res0 : r.res;
    std::fprintf(f,
                 "%s,%s,%s,%zu,%zu,%.17g,%s,%s,%s,%s,%s,%s,%.17g,%u,%d,"
                 "%zu,%zu,%zu,%zu,%zu,%zu,%zu,"
                 "%.9e,%.9e,%.9e,%.9e,%.9e,%.9e,%ld,%.9e,%d,%d,"
                 "%.17g,%zu,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g,%zu,%zu,%s\n",
                 a.phase.c_str(), a.problem.c_str(), a.family.c_str(), a.n, N, a.param, instance.c_str(),
                 method.c_str(), a.precond.c_str(), a.start.c_str(), start_id.c_str(), distance.c_str(), rho, seed,
                 r.converged ? 1 : 0, r.iters, r.n_F, r.n_JVP, r.n_D2, r.n_lin_iters, r.n_lin_failures, r.n_prec,
                 t_setup + r.raw.t_setup_dynamic, r.raw.t_F, r.raw.t_JVP, r.raw.t_D2, r.raw.t_prec, t_total,
                 max_rss_kb(), rel, 1, repetition, a.rtol, a.max_nl, a.eta_init, a.eta_max, a.gamma, a.alpha,
                 a.eta2_factor, a.eta2_max, a.restart, a.maxlin, a.commit.c_str());
    std::fclose(f);
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc == 2 && std::string(argv[1]) == "--print-header") {  // the CSV schema, no GPU needed
        std::printf("%s\n", kHeader);
        return 0;
    }
    Args a;
    if (!parse(argc, argv, a)) {
        std::fprintf(stderr,
                     "usage: %s --phase exploratory|calibration|confirmation --problem bratu --n N --param P "
                     "--precond mg|jacobi|none --methods nk,cheb,rec,tf2018 "
                     "--start natural|perturbed|continuation|coarse [--start-file vector.txt] [--start-id ID] "
                     "[--dist near,mid,far] [--seeds 12] [--warmup 1] [--reps 7] [--rtol 1e-8] [--max-nl 50] "
                     "[--eta-init 0.5] [--eta-max 0.9] [--gamma 0.9] [--alpha 2.0] [--eta2-factor 10] "
                     "[--eta2-max 0.5] [--restart 50] [--maxlin 500] [--device 0] [--mg-precision fp64|fp32] "
                     "[--jvp analytic|fd] --out file.csv [--commit SHA]\n",
                     argv[0]);
        return 2;
    }
    if (!(a.param >= 0.0)) {
        std::fprintf(stderr, "Bratu lambda must be non-negative.\n");
        return 2;
    }
    try {
        numa::gpu::Context ctx(a.device);
        numa_gpu_ctx_set_timing(ctx.get(), 1);
        numa::gpu::Bratu3D problem(ctx, a.n, a.param);
        const std::size_t N = problem.size();
        DVec reference;
        if (!a.start_file.empty() && !load_vector(a.start_file, N, reference)) {
            std::fprintf(stderr, "could not read a vector of %zu values from %s\n", N, a.start_file.c_str());
            return 3;
        }
        numa::gpu::KrylovParams p;
        p.rtol_nl = a.rtol;
        p.max_nl = a.max_nl;
        p.eta_init = a.eta_init;
        p.eta_max = a.eta_max;
        p.gamma = a.gamma;
        p.alpha = a.alpha;
        p.eta2_factor = a.eta2_factor;
        p.eta2_max = a.eta2_max;
        p.gmres_restart = a.restart;
        p.gmres_max_iters = a.maxlin;
        p.jvp_mode = a.jvp_mode;
        if (a.mg_precision == NUMA_GPU_FP32) {
            p.flexible = 1;
            p.jvp_precision = NUMA_GPU_FP32;
        }

        auto run = [&](const DVec& x0, const std::string& method, const std::string& distance, double rho,
                       unsigned seed) -> bool {
            const std::string sid = a.start == "natural" ? "natural" : a.start_id;
            for (int rep = -a.warmup + 1; rep <= a.reps; ++rep) {
                const auto t0 = std::chrono::steady_clock::now();
                // the provider is built per solve, as the reference's factory does (run_campaign.cpp:354-357)
                auto pc = a.precond == "mg" ? numa::gpu::Provider::poisson_mg(ctx, a.n, a.mg_precision)
                          : a.precond == "jacobi" ? numa::gpu::Provider::jacobi(problem)
                                                  : numa::gpu::Provider::identity(ctx);
                const double t_setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                numa::gpu::KrylovParams q = p;
                numa::gpu::KrylovResult r;
                if (method == "nk") r = numa::gpu::newton_krylov(problem, x0, q, &pc);
                else if (method == "tf2018") r = numa::gpu::tf_chebyshev_2018(problem, x0, q, &pc);
                else {
                    q.recycle = method == "rec" ? 1 : 0;
                    r = numa::gpu::chebyshev_inexact(problem, x0, q, &pc);
                }
                const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                if (rep >= 1 && !append_row(a, N, method, sid, distance, rho, seed, r, t_setup, total, rep)) {
                    std::fprintf(stderr, "could not write %s\n", a.out.c_str());
                    return false;
                }
            }
            return true;
        };

        const DVec natural(N, 0.0);
        for (const auto& method : split(a.methods)) {
            if (a.start == "natural") {
                if (!run(natural, method, "natural", 0.0, 0)) return 3;
            } else if (a.start == "continuation" || a.start == "coarse") {
                if (!run(reference, method, a.start, 0.0, 0)) return 3;
            } else {
                for (const auto& d : split(a.dist)) {
                    const double rho = rho_for(d);
                    for (unsigned seed = 1; seed <= a.seeds; ++seed) {
                        const DVec x0 = perturb(reference, rho, seed);
                        if (x0.empty()) return 3;
                        if (!run(x0, method, d, rho, seed)) return 3;
                    }
                }
            }
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "run_campaign_gpu: %s\n", e.what());
        return 4;
    }
    return 0;
}
