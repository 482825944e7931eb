// lbm_zsc.cpp -- host driver of the ZSC multiphase lattice Boltzmann run on
// liblbm_gb300.so: the counterpart of the reference's main program
// (src/main.cu:83-667), calling the GPU only through the library's C-ABI.
//
// Reads properties.in and discrete.in from the run directory (the reference's
// positional format, src/paramread.c:36-75), runs
//   init -> relaxation (grav = 0, relaxStep steps) -> evolution (maxStep - 1 steps)
// and writes the reference's outputs into the same directory, at the same
// points of the run and in the same formats:
//   runlog.out                     src/logsave.c:181-279 (header, relaxation
//                                  results, output results, timing)
//   relax_stats.out, stats.out     src/stats.c:60-91 (a line every `stat` steps
//                                  and at the phase boundaries)
//   relax_data_00_NNNNNNN.vtk,     src/vtksave.c:29-145 (every `save` steps and
//   data_00_NNNNNNN.vtk            at the phase boundaries)
// Like the reference it keeps host copies of phi, rho and u and refreshes them
// where it does (phi and u at stat steps, all five at save steps and at the
// phase boundaries, src/main.cu:457-472, :481-490, :592-607, :627-632); the
// relaxation results of runlog.out are computed from those copies
// (src/main.cu:475-476 logs before refreshing them).  Statistics are FP64 reductions on the GPU.
//
// With --adjoint OBJECTIVE the run is instead the gradient of a light-phase
// objective over --adjoint-steps steps of evolution from the initial state
// (lbm_step_adjoint; no counterpart in the reference): J, dJ/dgrav and the
// schedule go to adjoint.out, dJ/dphi0 to adjoint_dphi0.vtk (binary).
//
// Usage: lbm_zsc [DIR] [--storage fp32|fp16|bf16] [--vtk ascii|binary|none]
//                [--device N] [--no-compat]
//                [--adjoint light_uz_mean|light_z_centroid --adjoint-steps T
//                 --adjoint-window W --checkpoint-gb G]
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "lbm_gb300.h"

namespace {

constexpr double kMB = 1048576.0;
constexpr double kGB = 1073741824.0;

struct Options {
    std::string dir = ".";
    int storage = LBM_STORAGE_FP32;
    int vtk = 1;   // 0 none, 1 ASCII (the reference's format), 2 binary legacy VTK
    int device = 0;
    int compat = 1;
    int adjoint = -1;          // LBM_OBJ_*, -1: the reference's run
    int adjoint_steps = 1000;
    int adjoint_window = 1;
    double checkpoint_gb = 0.0;   // <= 0: the library's default (free device memory less a reserve)
};

[[noreturn]] void fatal(const std::string &what, int code)
{
    std::fprintf(stderr, "ERROR: %s: %s (%s).\n", what.c_str(), lbm_strerror(code), lbm_last_error());
    std::exit(1);
}

void check(int code, const char *what)
{
    if (code != LBM_OK) fatal(what, code);
}

void usage(const char *argv0)
{
    std::printf("usage: %s [DIR] [--storage fp32|fp16|bf16] [--vtk ascii|binary|none] [--device N] [--no-compat]\n"
                "       [--adjoint light_uz_mean|light_z_centroid [--adjoint-steps T] [--adjoint-window W]\n"
                "        [--checkpoint-gb G]]\n"
                "Runs the ZSC multiphase LBM described by DIR/properties.in and DIR/discrete.in\n"
                "(default DIR: the current directory) and writes runlog.out, relax_stats.out,\n"
                "stats.out and the VTK snapshots into DIR.  With --adjoint it computes the\n"
                "gradient of the objective over T evolution steps from the initial state\n"
                "instead (adjoint.out, adjoint_dphi0.vtk).\n",
                argv0);
}

Options parse(int argc, char **argv)
{
    Options o;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        auto value = [&]() -> std::string {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "ERROR: %s needs a value.\n", a.c_str());
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "-h" || a == "--help") {
            usage(argv[0]);
            std::exit(0);
        } else if (a == "--storage") {
            const std::string v = value();
            o.storage = v == "fp32" ? LBM_STORAGE_FP32 : v == "fp16" ? LBM_STORAGE_FP16 : v == "bf16" ? LBM_STORAGE_BF16 : -1;
            if (o.storage < 0) {
                std::fprintf(stderr, "ERROR: unknown storage '%s'.\n", v.c_str());
                std::exit(2);
            }
        } else if (a == "--vtk") {
            const std::string v = value();
            o.vtk = v == "none" ? 0 : v == "ascii" ? 1 : v == "binary" ? 2 : -1;
            if (o.vtk < 0) {
                std::fprintf(stderr, "ERROR: unknown VTK mode '%s'.\n", v.c_str());
                std::exit(2);
            }
        } else if (a == "--device") {
            o.device = std::atoi(value().c_str());
        } else if (a == "--no-compat") {
            o.compat = 0;
        } else if (a == "--adjoint") {
            const std::string v = value();
            o.adjoint = v == "light_uz_mean" ? LBM_OBJ_LIGHT_UZ_MEAN : v == "light_z_centroid" ? LBM_OBJ_LIGHT_Z_CENTROID : -2;
            if (o.adjoint < -1) {
                std::fprintf(stderr, "ERROR: unknown objective '%s'.\n", v.c_str());
                std::exit(2);
            }
        } else if (a == "--adjoint-steps") {
            o.adjoint_steps = std::atoi(value().c_str());
        } else if (a == "--adjoint-window") {
            o.adjoint_window = std::atoi(value().c_str());
        } else if (a == "--checkpoint-gb") {
            o.checkpoint_gb = std::atof(value().c_str());
        } else if (!a.empty() && a[0] == '-') {
            std::fprintf(stderr, "ERROR: unknown option '%s'.\n", a.c_str());
            usage(argv[0]);
            std::exit(2);
        } else {
            o.dir = a;
        }
    }
    return o;
}

std::string stamp(const char *fmt)
{
    char buf[32];
    const std::time_t t = std::time(nullptr);
    std::strftime(buf, sizeof(buf), fmt, std::localtime(&t));
    return buf;
}

struct Host {
    size_t n = 0;
    std::vector<float> phi, rho, ux, uy, uz;
    explicit Host(size_t n_) : n(n_), phi(n_), rho(n_), ux(n_), uy(n_), uz(n_) {}
};

class Run {
public:
    Run(const Options &o) : o_(o) {}

    int main()
    {
        const auto t_start = clock();
        read_inputs();
        check(lbm_device_name(o_.device, dev_name_, sizeof(dev_name_), &dev_mem_), "lbm_device_name");
        banner();
        check(lbm_init_bubbles(&c_, &p_, bubbles_.data(), nbubbles_), "lbm_init_bubbles");
        check(lbm_derive(&p_, &d_), "lbm_derive");
        if (o_.adjoint >= 0) return adjoint();
        host_ = new Host((size_t)p_.nx * p_.ny * p_.nz);
        lbm_stats_out s = copy_fields(true);

        // setup (src/main.cu:294-358)
        log_header();
        relax_ = 1;
        step_ = 0;
        stats_line(s, true);
        vtk_save();
        std::printf("Data initialization completed.\n");
        check(lbm_sync(c_), "lbm_sync");
        const auto t_setup = clock();

        // relaxation (src/main.cu:360-492)
        loop(1, run_.relax_step, 0.f);
        log_relaxation();
        std::printf("Relaxation run completed.\n");
        relax_ = 0;
        s = copy_fields(true);
        step_ = 0;
        stats_line(s, true);
        vtk_save();
        check(lbm_sync(c_), "lbm_sync");
        const auto t_relax = clock();

        // evolution (src/main.cu:494-626)
        std::printf("Starting evolution run ...\n");
        loop(1, run_.max_step - 1, d_.grav);
        step_ = run_.max_step;
        std::printf("Evolution run completed.\n");
        check(lbm_sync(c_), "lbm_sync");
        const auto t_main = clock();

        setup_ms_ = ms(t_start, t_setup);
        relax_ms_ = ms(t_setup, t_relax);
        main_ms_ = ms(t_relax, t_main);
        const double total_ms = ms(t_start, t_main);
        std::printf("Setup time      : %6.3f ms\n", setup_ms_);
        std::printf("Relaxation time : %6.3f ms\n", relax_ms_);
        std::printf("Evolution time  : %6.3f ms\n", main_ms_);
        std::printf("Total time      : %6.3f ms\n", total_ms);
        std::printf("Time for lb step: %6.3f ms\n", run_.max_step > 0 ? main_ms_ / run_.max_step : 0.0);
        const long long evolved = run_.max_step > 1 ? run_.max_step - 1 : 0;
        if (evolved > 0)
            std::printf("Measured MLUPS  : %.1f (%lld steps of %lld nodes)\n",
                        (double)evolved * (double)host_->n / (main_ms_ * 1e3), evolved, (long long)host_->n);

        // final output (src/main.cu:627-637)
        s = copy_fields(true);
        log_output(s);
        stats_line(s, false);
        vtk_save();
        lbm_destroy(c_);
        delete host_;
        return 0;
    }

private:
    using Clock = std::chrono::steady_clock;
    static Clock::time_point clock() { return Clock::now(); }
    static double ms(Clock::time_point a, Clock::time_point b)
    {
        return std::chrono::duration<double, std::milli>(b - a).count();
    }

    // the gradient run (no counterpart in the reference)
    int adjoint()
    {
        const size_t n = (size_t)p_.nx * p_.ny * p_.nz;
        std::vector<float> grad(n);
        lbm_adjoint_opts o{};
        o.objective = o_.adjoint;
        o.nsteps = o_.adjoint_steps;
        o.window = o_.adjoint_window;
        o.grav = d_.grav;
        o.checkpoint_bytes = o_.checkpoint_gb * 1e9;
        lbm_adjoint_out r{};
        r.dJ_dphi0 = grad.data();
        check(lbm_step_adjoint(c_, &o, &r), "lbm_step_adjoint");
        FILE *fp = open("adjoint.out", "w");
        std::fprintf(fp, "objective          = %s\n", o.objective == LBM_OBJ_LIGHT_UZ_MEAN ? "light_uz_mean" : "light_z_centroid");
        std::fprintf(fp, "steps              = %d\n", o.nsteps);
        std::fprintf(fp, "window             = %d\n", o.window);
        std::fprintf(fp, "grav               = %e\n", (double)o.grav);
        std::fprintf(fp, "J                  = %.17e\n", r.J);
        std::fprintf(fp, "dJ/dgrav           = %.17e\n", r.dJ_dgrav);
        std::fprintf(fp, "checkpoint slots   = %d\n", r.slots);
        std::fprintf(fp, "checkpoint GB      = %.3f\n", r.checkpoint_bytes_used / 1e9);
        std::fprintf(fp, "forward steps      = %lld\n", r.forward_steps);
        std::fprintf(fp, "adjoint steps      = %lld\n", r.adjoint_steps);
        std::fprintf(fp, "seconds            = %.6f\n", r.seconds);
        std::fclose(fp);
        std::printf("J = %.10e  dJ/dgrav = %.10e  (%d slots, %lld forward steps, %.3f s)\n", r.J, r.dJ_dgrav, r.slots,
                    r.forward_steps, r.seconds);
        fp = open("adjoint_dphi0.vtk", "wb");
        std::fprintf(fp, "# vtk DataFile Version 2.0\n");
        std::fprintf(fp, "dJ/dphi0 (liblbm_gb300 adjoint)\nBINARY\n\nDATASET STRUCTURED_POINTS\n");
        std::fprintf(fp, "DIMENSIONS %d %d %d\nORIGIN 1 1 1\nSPACING 1 1 1\n\nPOINT_DATA %lld\n\n", p_.nx, p_.ny, p_.nz,
                     (long long)n);
        std::fprintf(fp, "SCALARS dJ_dphi0 float\nLOOKUP_TABLE default\n");
        put_be(fp, grad.data(), n);
        std::fprintf(fp, "\n");
        std::fclose(fp);
        lbm_destroy(c_);
        return 0;
    }

    void read_inputs()
    {
        std::vector<float> buf(4 * 4096);
        int count = 0;
        check(lbm_read_inputs(o_.dir.c_str(), &p_, &run_, buf.data(), 4096, &count), "reading the input files");
        if (count > 4096) {
            buf.assign(4 * (size_t)count, 0.f);
            check(lbm_read_inputs(o_.dir.c_str(), &p_, &run_, buf.data(), count, &count), "reading the input files");
        }
        nbubbles_ = count;
        bubbles_.assign(buf.begin(), buf.begin() + 4 * (size_t)count);
        p_.storage = o_.storage;
        p_.device = o_.device;
        p_.compat = o_.compat;
    }

    void banner()
    {
        std::printf("*** Multiphase Zheng-Shu-Chew LBM 3D Simulation \n");
        std::printf("*** GB300 fused-step implementation (liblbm_gb300)\n\n");
        std::printf("*** Program running on : %s\n", dev_name_);
        if (dev_mem_ >= kGB)
            std::printf("*** Total GPU Memory   : %.4f GB\n\n", dev_mem_ / kGB);
        else
            std::printf("*** Total GPU Memory   : %.4f MB\n\n", dev_mem_ / kMB);
    }

    std::string path(const std::string &name) const { return o_.dir + "/" + name; }

    FILE *open(const std::string &name, const char *mode) const
    {
        FILE *fp = std::fopen(path(name).c_str(), mode);
        if (!fp) {
            std::fprintf(stderr, "ERROR: cannot open %s.\n", path(name).c_str());
            std::exit(1);
        }
        return fp;
    }

    // Host copies: phi and u always, rho when `all` (src/main.cu:457-472),
    // with the statistics of the current fields (which the refreshed copies
    // of phi and u equal; the statistics do not read rho apart from the
    // pressure sums, which only the runlog reports).
    lbm_stats_out copy_fields(bool all)
    {
        Host &h = *host_;
        lbm_stats_out s;
        check(lbm_stats(c_, &s, h.phi.data(), all ? h.rho.data() : nullptr, h.ux.data(), h.uy.data(), h.uz.data()),
              "lbm_stats");
        return s;
    }

    // steps first..last with output at the stat and save multiples
    void loop(long long first, long long last, float grav)
    {
        long long s = first;
        while (s <= last) {
            long long next = last;
            if (run_.stat > 0) next = std::min(next, ((s + run_.stat - 1) / run_.stat) * run_.stat);
            if (run_.save > 0) next = std::min(next, ((s + run_.save - 1) / run_.save) * run_.save);
            check(lbm_step(c_, (int)(next - s + 1), grav), "lbm_step");
            step_ = next;
            if (run_.stat > 0 && next % run_.stat == 0) stats_line(copy_fields(false), false);
            if (run_.save > 0 && next % run_.save == 0) {
                copy_fields(true);
                vtk_save();
            }
            s = next + 1;
        }
    }

    lbm_stats_out host_stats() const
    {
        lbm_stats_out s;
        const Host &h = *host_;
        check(lbm_stats_fields(c_, &s, h.phi.data(), h.rho.data(), h.ux.data(), h.uy.data(), h.uz.data()),
              "lbm_stats_fields");
        return s;
    }

    // src/stats.c:60-91
    void stats_line(const lbm_stats_out &s, bool first)
    {
        const char *name = relax_ == 0 ? "stats.out" : "relax_stats.out";
        if (first) {
            if (relax_ == 0)
                inv_init_vol_ = 1.0 / s.vol;
            else
                inv_relax_vol_ = 1.0 / s.vol;
            FILE *fp = open(name, "w");
            std::fprintf(fp, "#step\t\tux\t\tuy\t\tuz\t\tUmax\t\tVef\t\tRef\n");
            std::fclose(fp);
        }
        const double vef = s.vol * (relax_ == 0 ? inv_init_vol_ : inv_relax_vol_);
        FILE *fp = open(name, "a");
        std::fprintf(fp, "%8lld\t%e\t%e\t%e\t%e\t%e\t%e\n", (long long)step_, s.ux_av, s.uy_av, s.uz_av, s.umax, vef,
                     s.ref);
        std::fclose(fp);
    }

    void memory(double &dist, double &aux, double &cpu, double &gpu) const
    {
        const double n = (double)host_->n;
        const double esz = p_.storage == LBM_STORAGE_FP32 ? 4.0 : 2.0;
        dist = 2.0 * 4.0 * n + 2.0 * 6.0 * esz * n + 19.0 * esz * n;   // f_0, f_1..f_6 (A/B), g (AA)
        aux = 5.0 * 4.0 * n;                                            // phi, rho, u on the device
        cpu = 5.0 * 4.0 * n;                                            // their host copies
        gpu = dist + aux;
    }

    // src/logsave.c:181-240
    void log_header()
    {
        FILE *fp = open("runlog.out", "w");
        std::fprintf(fp, "***\n");
        std::fprintf(fp, "*** Multiphase Zheng-Shu-Chew LBM 3D Simulation  \n");
        std::fprintf(fp, "*** GB300 fused-step implementation (liblbm_gb300) \n");
        std::fprintf(fp, "***\n");
        std::fprintf(fp, "*** Program running on : %s\n", dev_name_);
        if (dev_mem_ >= kGB)
            std::fprintf(fp, "*** Total GPU Memory   : %.4f GB\n", dev_mem_ / kGB);
        else
            std::fprintf(fp, "*** Total GPU Memory   : %.4f MB\n", dev_mem_ / kMB);
        std::fprintf(fp, "***\n");
        std::fprintf(fp, "*** Simulation started at %s on %s\n", stamp("%H:%M").c_str(), stamp("%Y-%m-%d").c_str());
        std::fprintf(fp, "***\n\n");

        std::fprintf(fp, "INPUT PARAMETERS\n");
        std::fprintf(fp, "Evolution Steps    = %d\n", run_.max_step);
        std::fprintf(fp, "Relaxation Steps   = %d\n", run_.relax_step);
        std::fprintf(fp, "Domain Size in X   = %d\n", p_.nx);
        std::fprintf(fp, "Domain Size in Y   = %d\n", p_.ny);
        std::fprintf(fp, "Domain Size in Z   = %d\n", p_.nz);
        std::fprintf(fp, "Interface Width    = %6.3f\n", p_.width);
        std::fprintf(fp, "Interface Tension  = %6.3f\n", p_.sigma);
        std::fprintf(fp, "Interface Mobility = %6.3f\n", p_.Gamma);
        std::fprintf(fp, "Low Fluid Density  = %6.3f\n", p_.rhoL);
        std::fprintf(fp, "High Fluid Density = %6.3f\n", p_.rhoH);
        std::fprintf(fp, "Tau (Density)      = %6.3f\n", p_.tauRho);
        std::fprintf(fp, "Tau (Phase)        = %6.3f\n", p_.tauPhi);
        std::fprintf(fp, "\n");

        std::fprintf(fp, "CUDA CONFIGURATION\n");
        std::fprintf(fp, "GPUs used    = %d\n", 1);
        std::fprintf(fp, "BLOCK_SIZE_X = %d\n", p_.block_x);
        std::fprintf(fp, "BLOCK_SIZE_Y = %d\n", p_.block_y);
        std::fprintf(fp, "\n");

        double dist, aux, cpu, gpu;
        memory(dist, aux, cpu, gpu);
        const bool gb = gpu >= kGB;
        const double unit = gb ? kGB : kMB;
        std::fprintf(fp, gb ? "MEMORY USAGE (Gb)\n" : "MEMORY USAGE (Mb)\n");
        std::fprintf(fp, "Distributions         = %4.2f\n", dist / unit);
        std::fprintf(fp, "Auxiliary Arrays      = %4.2f\n", aux / unit);
        std::fprintf(fp, "Total CPU Memory Used = %4.2f\n", cpu / unit);
        std::fprintf(fp, "Total GPU Memory Used = %4.2f\n", gpu / unit);
        std::fprintf(fp, "\n");
        std::fclose(fp);
    }

    // src/logsave.c:241-252; "Parasitic Velocity" is max |u|^2 there
    void log_relaxation()
    {
        const lbm_stats_out s = host_stats();
        FILE *fp = open("runlog.out", "a");
        std::fprintf(fp, "RELAXATION RESULTS\n");
        std::fprintf(fp, "Effective Radius   = %e\n", s.ref);
        std::fprintf(fp, "Phase Conservation = %e\n", s.vol * inv_relax_vol_);
        std::fprintf(fp, "(Pin - Pout)       = %e\n", s.p_dif);
        std::fprintf(fp, "Laplace Error      = %e\n", s.p_err);
        std::fprintf(fp, "Parasitic Velocity = %e\n", s.umax * s.umax);
        std::fprintf(fp, "\n");
        std::fclose(fp);
    }

    // src/logsave.c:253-279.  The MLUPS line keeps the reference's formula:
    // maxStep steps of NX*NY*(NZ+2) nodes (its grid with the two ghost planes).
    void log_output(const lbm_stats_out &s)
    {
        FILE *fp = open("runlog.out", "a");
        std::fprintf(fp, "OUTPUT RESULTS\n");
        std::fprintf(fp, "Effective Radius   = %e\n", s.ref);
        std::fprintf(fp, "Phase Conservation = %e\n", s.vol * inv_init_vol_);
        std::fprintf(fp, "Maximum Velocity   = %e\n", s.umax * s.umax);
        std::fprintf(fp, "\n");
        const double grid = (double)p_.nx * p_.ny * (p_.nz + 2);
        const double lbstep = run_.max_step > 0 ? main_ms_ * 1e-3 / run_.max_step : 0.0;
        const double mlups = main_ms_ > 0 ? (double)run_.max_step * grid * 1e-6 / (main_ms_ * 1e-3) : 0.0;
        std::fprintf(fp, "TIMING INFORMATION (seconds)\n");
        std::fprintf(fp, "Setup Time      = %9.6f\n", setup_ms_ * 1e-3);
        std::fprintf(fp, "Relaxation Time = %9.6f\n", relax_ms_ * 1e-3);
        std::fprintf(fp, "Main Loop Time  = %9.6f\n", main_ms_ * 1e-3);
        std::fprintf(fp, "LBM step Time   = %9.6f\n", lbstep);
        std::fprintf(fp, "MLUPS           = %9.6f\n", mlups);
        std::fprintf(fp, "\n");
        std::fprintf(fp, "***\n");
        std::fprintf(fp, "*** Simulation completed at %s on %s\n", stamp("%H:%M").c_str(), stamp("%Y-%m-%d").c_str());
        std::fprintf(fp, "***\n");
        std::fclose(fp);
    }

    static void put_be(FILE *fp, const float *v, size_t count)
    {
        std::vector<unsigned char> buf(4 * count);
        for (size_t i = 0; i < count; i++) {
            uint32_t u;
            std::memcpy(&u, &v[i], 4);
            buf[4 * i] = (unsigned char)(u >> 24);
            buf[4 * i + 1] = (unsigned char)(u >> 16);
            buf[4 * i + 2] = (unsigned char)(u >> 8);
            buf[4 * i + 3] = (unsigned char)u;
        }
        std::fwrite(buf.data(), 1, buf.size(), fp);
    }

    // src/vtksave.c:29-145: phi, pressure and velocity of the host copies,
    // legacy structured points; ASCII with "%f" as the reference, or binary
    // (big-endian float32) for large boxes.  The pressure is computed on the
    // GPU from the current phi and rho, which the host copies equal at every
    // point where a snapshot is written.
    void vtk_save()
    {
        if (o_.vtk == 0) return;
        const Host &h = *host_;
        std::vector<float> pres(h.n);
        check(lbm_pressure(c_, pres.data()), "lbm_pressure");
        char name[64];
        std::snprintf(name, sizeof(name), relax_ == 0 ? "data_%02d_%07lld.vtk" : "relax_data_%02d_%07lld.vtk", 0,
                      (long long)step_);
        FILE *fp = open(name, o_.vtk == 2 ? "wb" : "w");
        const bool bin = o_.vtk == 2;
        std::fprintf(fp, "# vtk DataFile Version 2.0\n");
        std::fprintf(fp, "ZSC multiphase LBM (liblbm_gb300)\n");
        std::fprintf(fp, bin ? "BINARY\n" : "ASCII\n");
        std::fprintf(fp, "\n");
        std::fprintf(fp, "DATASET STRUCTURED_POINTS\n");
        std::fprintf(fp, "DIMENSIONS %d %d %d\n", p_.nx, p_.ny, p_.nz);
        std::fprintf(fp, "ORIGIN %d %d %d\n", 1, 1, 1);
        std::fprintf(fp, "SPACING %d %d %d\n", 1, 1, 1);
        std::fprintf(fp, "\n");
        std::fprintf(fp, "POINT_DATA %lld\n", (long long)h.n);
        std::fprintf(fp, "\n");
        std::fprintf(fp, "SCALARS Phi float\n");
        std::fprintf(fp, "LOOKUP_TABLE default\n");
        if (bin) {
            put_be(fp, h.phi.data(), h.n);
        } else {
            for (size_t i = 0; i < h.n; i++) std::fprintf(fp, "%f\n", h.phi[i]);
        }
        std::fprintf(fp, "\n");
        std::fprintf(fp, "SCALARS Pressure float\n");
        std::fprintf(fp, "LOOKUP_TABLE default\n");
        if (bin) {
            put_be(fp, pres.data(), h.n);
        } else {
            for (size_t i = 0; i < h.n; i++) std::fprintf(fp, "%f\n", pres[i]);
        }
        std::fprintf(fp, "\n");
        if (bin) {
            std::fprintf(fp, "VECTORS Velocity float\n");
            std::vector<float> v(3 * h.n);
            for (size_t i = 0; i < h.n; i++) {
                v[3 * i] = h.ux[i];
                v[3 * i + 1] = h.uy[i];
                v[3 * i + 2] = h.uz[i];
            }
            put_be(fp, v.data(), v.size());
            std::fprintf(fp, "\n");
        } else {
            std::fprintf(fp, "Vectors Velocity float\n");
            for (size_t i = 0; i < h.n; i++) std::fprintf(fp, "%f %f %f\n", h.ux[i], h.uy[i], h.uz[i]);
        }
        std::fclose(fp);
    }

    Options o_;
    lbm_params p_{};
    lbm_run run_{};
    lbm_derived d_{};
    std::vector<float> bubbles_;
    int nbubbles_ = 0;
    lbm_ctx *c_ = nullptr;
    Host *host_ = nullptr;
    char dev_name_[256] = {0};
    double dev_mem_ = 0.0;
    int relax_ = -1;
    long long step_ = 0;
    double inv_init_vol_ = 0.0, inv_relax_vol_ = 0.0;
    double setup_ms_ = 0.0, relax_ms_ = 0.0, main_ms_ = 0.0;
};

}  // namespace

int main(int argc, char **argv)
{
    const Options o = parse(argc, argv);
    return Run(o).main();
}
