// s2d_driver.cpp -- the Spectral2D main program on the GB300 library.
//
// Host-side counterpart of src/Spectral2D.F90: the same run parameters (as
// command-line options instead of compile-time PARAMETERs, :70-127), the same
// set-up order (grid, IC, restart 0, Analysis at nadv = 0), and the same time
// loop (:338-432) with its print / write / stat cadences -- including the
// reference's look-ahead flags (an event fires on the step after
// nadv + 1 == *Step was seen) and the DESIRED_END_TIME dt adjustment.  Output
// follows the reference's formats: the step line (:371-377), EULERIAN.DAT
// (src/Analysis.F90:47-54, :237-240), SPECTRUM_<nadv>.DAT
// (src/Analysis.F90:424-434) and REST_<num> restart files.  Steps between
// events are replayed from the library's CUDA graph.
#include "s2d.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int FIXED_STEP_COUNT = 1;   // src/Spectral2D.F90:66
constexpr int DESIRED_END_TIME = 2;   // src/Spectral2D.F90:68
constexpr int TAYLOR_GREEN_VORTEX = 1;      // src/SetIC.F90:35
constexpr int SCHUMANN_VELOCITY_FIELD = 2;  // src/SetIC.F90:37
constexpr int K4_GAUSS_FIELD = 3;           // the decaying-turbulence spectrum

struct Params {
    int nx = 96, ny = 96;             // :73-75
    double nu = 0.005;                // :80
    int endMethod = FIXED_STEP_COUNT; // :89
    long stepEnd = 2000000;           // :94
    double dt = 1.0e-5;               // :96
    double tEnd = 1.0;                // :101
    long writePeriod = 10000;         // :106
    long statPeriod = 1000;           // :108
    long printPeriod = 10;            // :110
    int ics = SCHUMANN_VELOCITY_FIELD;  // :115
    double k0 = 1.5, urms = 1.0;      // :120-122
    double tke = 0.0;                 // 0: no rescale (the reference's behaviour)
    uint64_t seed = 0;
    double cfl = 0.0;                 // > 0: dt from CFL of the initial condition
    int precision = S2D_FP64;
    std::string out = ".";
    std::string statRoot = "EULERIAN";   // :127
    std::string resume, checkpoint;
};

void usage() {
    std::fprintf(stderr,
                 "spectral2d_run [--nx N] [--ny N] [--nu NU] [--dt DT] [--steps N | --end-time T]\n"
                 "  [--cfl C] [--ic tg|schumann|k4gauss] [--k0 K0] [--urms U] [--tke E] [--seed S]\n"
                 "  [--print-period N] [--stat-period N] [--write-period N] [--precision fp64|fp32]\n"
                 "  [--out DIR] [--resume CKPT] [--checkpoint CKPT]\n"
                 "  (--nx sets ny too unless --ny is given)\n");
}

// --nx sets both sizes (the library runs square grids) unless --ny is given.
bool parse(int argc, char** argv, Params& p) {
    bool ny_given = false;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto val = [&](const char* name) -> const char* {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "missing value for %s\n", name);
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "--nx") p.nx = std::atoi(val("--nx"));
        else if (a == "--ny") { p.ny = std::atoi(val("--ny")); ny_given = true; }
        else if (a == "--nu") p.nu = std::atof(val("--nu"));
        else if (a == "--dt") p.dt = std::atof(val("--dt"));
        else if (a == "--steps") { p.stepEnd = std::atol(val("--steps")); p.endMethod = FIXED_STEP_COUNT; }
        else if (a == "--end-time") { p.tEnd = std::atof(val("--end-time")); p.endMethod = DESIRED_END_TIME; }
        else if (a == "--cfl") p.cfl = std::atof(val("--cfl"));
        else if (a == "--ic") {
            const std::string v = val("--ic");
            if (v == "tg") p.ics = TAYLOR_GREEN_VORTEX;
            else if (v == "schumann") p.ics = SCHUMANN_VELOCITY_FIELD;
            else if (v == "k4gauss") p.ics = K4_GAUSS_FIELD;
            else return false;
        } else if (a == "--k0") p.k0 = std::atof(val("--k0"));
        else if (a == "--urms") p.urms = std::atof(val("--urms"));
        else if (a == "--tke") p.tke = std::atof(val("--tke"));
        else if (a == "--seed") p.seed = std::strtoull(val("--seed"), nullptr, 10);
        else if (a == "--print-period") p.printPeriod = std::atol(val("--print-period"));
        else if (a == "--stat-period") p.statPeriod = std::atol(val("--stat-period"));
        else if (a == "--write-period") p.writePeriod = std::atol(val("--write-period"));
        else if (a == "--precision") p.precision = std::string(val("--precision")) == "fp32" ? S2D_FP32 : S2D_FP64;
        else if (a == "--out") p.out = val("--out");
        else if (a == "--resume") p.resume = val("--resume");
        else if (a == "--checkpoint") p.checkpoint = val("--checkpoint");
        else return false;
    }
    if (!ny_given) p.ny = p.nx;
    return p.printPeriod > 0 && p.statPeriod > 0 && p.writePeriod > 0;
}

#define CHECK(call)                                                                       \
    do {                                                                                  \
        const int r_ = (call);                                                            \
        if (r_ != S2D_OK) {                                                               \
            std::fprintf(stderr, "%s failed (%d): %s\n", #call, r_, s2d_last_error());    \
            std::exit(1);                                                                 \
        }                                                                                 \
    } while (0)

// Text with each field starting at a 1-based column (Fortran T edit descriptor).
std::string tabbed(const std::vector<std::pair<int, const char*>>& fields) {
    std::string s;
    for (const auto& f : fields) {
        while ((int)s.size() < f.first - 1) s += ' ';
        s += f.second;
    }
    return s;
}

struct Run {
    Params p;
    s2d_handle* h = nullptr;
    long nadv = 0;
    double time = 0.0;
    double dt = 0.0;
    long pending = 0;   // steps issued to the GPU lazily
    int restNum = 0;    // src/IO.F90:45
    std::string eulOut;

    void flush() {
        if (pending > 0) CHECK(s2d_integrate_steps(h, (int32_t)pending, dt));
        pending = 0;
    }

    // src/IO.F90:98-143 (physical fields, here with an XDMF sidecar)
    void write_restart() {
        flush();
        std::printf("Writing REST_%06d.bin at t = %15.8E and nadv = %08ld\n", restNum, time, nadv);
        CHECK(s2d_write_restart(h, (p.out + "/REST").c_str(), restNum, nadv, time));
        restNum += 1;
    }

    // src/Analysis.F90:39-58
    void setup_analysis() {
        eulOut = p.out + "/" + p.statRoot + ".DAT";
        FILE* f = std::fopen(eulOut.c_str(), "w");
        if (!f) {
            std::fprintf(stderr, "cannot open %s\n", eulOut.c_str());
            std::exit(1);
        }
        std::fprintf(f, "%s\n",
                     tabbed({{1, "#"}, {3, "NADV"}, {17, "TIME"}, {33, "TKE"}, {49, "EPS"}, {65, "EnstDiss"},
                             {81, "xSkew"}, {97, "ySkew"}})
                         .c_str());
        std::fclose(f);
    }

    // src/Analysis.F90:90-242 and ComputeSpectrum's file (:423-435)
    void analysis() {
        flush();
        std::printf("Writing Eulerian statistics at t = %15.8E and nadv = %08ld\n", time, nadv);
        double xs = 0, ys = 0, tke = 0, eps = 0, enst = 0;
        CHECK(s2d_skewness(h, &xs, &ys));
        const int nb = s2d_spectrum_bins(h);
        std::vector<double> Ek(nb);
        CHECK(s2d_spectrum(h, Ek.data(), nb, &tke, &eps, &enst));
        char name[64];
        std::snprintf(name, sizeof(name), "/SPECTRUM_%08ld.DAT", nadv);
        FILE* f = std::fopen((p.out + name).c_str(), "w");
        if (f) {
            std::fprintf(f, "%s\n", tabbed({{1, "#"}, {3, "k"}, {11, "E(k)"}, {28, "D(k)"}, {45, "DEnst(k)"}}).c_str());
            for (int i = 0; i < nb; ++i) {
                const double k = (double)i;
                std::fprintf(f, "%6.6d%16.8E %16.8E %16.8E\n", i, Ek[i], k * k * Ek[i], k * k * k * k * Ek[i]);
            }
            std::fclose(f);
        }
        f = std::fopen(eulOut.c_str(), "a");
        if (f) {
            std::fprintf(f, "%12.10ld%16.8E%16.8E%16.8E%16.8E%16.8E%16.8E\n", nadv, time, tke, eps, enst, xs, ys);
            std::fclose(f);
        }
    }

    // src/Spectral2D.F90:357-377
    void print_step() {
        flush();
        double mm[4];
        CHECK(s2d_minmax_abs(h, mm));
        std::printf("Simulation step number: %08ld; Simulation time: %15.8E; Max W: %15.8E; Min W: %15.8E; "
                    "Max Psi: %15.8E; Min Psi: %15.8E\n",
                    nadv, time, mm[0], mm[1], mm[2], mm[3]);
    }
};

}  // namespace

int main(int argc, char** argv) {
    Run run;
    Params& p = run.p;
    if (!parse(argc, argv, p)) {
        usage();
        return 2;
    }
    s2d_config cfg{};
    cfg.nx = p.nx;
    cfg.ny = p.ny;
    cfg.dealias = S2D_DEALIAS_3_2_RULE;
    cfg.precision = p.precision;
    cfg.nu = p.nu;
    cfg.nonlinear_form = S2D_NL_BASDEVANT;
    CHECK(s2d_create(&cfg, &run.h));   // GetGridSize ... SetupPlans (:263-307)
    s2d_grid g;
    CHECK(s2d_get_grid_size(p.nx, p.ny, S2D_DEALIAS_3_2_RULE, &g));
    std::printf("Grid %d x %d (collocation %d x %d), nu = %15.8E\n", p.nx, p.ny, g.nxG, g.nyG, p.nu);

    // initial conditions (:310-319) or a checkpoint
    if (!p.resume.empty()) {
        int64_t n = 0;
        CHECK(s2d_checkpoint_read(run.h, p.resume.c_str(), &n, &run.time));
        run.nadv = (long)n;
    } else if (p.ics == TAYLOR_GREEN_VORTEX) {
        CHECK(s2d_set_taylor_green(run.h));
    } else {
        const int spec = p.ics == K4_GAUSS_FIELD ? S2D_SPECTRUM_K4_GAUSS : S2D_SPECTRUM_SCHUMANN;
        CHECK(s2d_set_turbulent(run.h, p.seed, spec, p.k0, p.urms, p.tke));
    }
    run.dt = p.dt;
    if (p.cfl > 0.0) CHECK(s2d_cfl_dt(run.h, p.cfl, &run.dt));

    run.write_restart();     // :322-324
    run.setup_analysis();    // :327
    run.analysis();          // :328-330

    // time loop (:333-432)
    bool loopBool = true, exitThisStep = false, writeBool = false, statBool = false, printBool = false;
    long writeStep = run.nadv + p.writePeriod, statStep = run.nadv + p.statPeriod, printStep = run.nadv + p.printPeriod;
    if (p.endMethod == FIXED_STEP_COUNT && run.nadv + 1 >= p.stepEnd) exitThisStep = true;
    while (loopBool) {
        run.pending += 1;        // IntegrateOneStep (:342-343), issued lazily
        run.time = run.time + run.dt;
        run.nadv = run.nadv + 1;
        // ComputeTimeStep (:350) is an empty stub in the reference
        if (printBool || exitThisStep) {
            printStep = printStep + p.printPeriod;
            printBool = false;
            run.print_step();
        } else if (run.nadv + 1 == printStep) {
            printBool = true;
        }
        if (writeBool || exitThisStep) {
            writeStep = writeStep + p.writePeriod;
            writeBool = false;
            run.write_restart();
        } else if (run.nadv + 1 == writeStep) {
            writeBool = true;
        }
        if (statBool || exitThisStep) {
            statStep = statStep + p.statPeriod;
            statBool = false;
            run.analysis();
        } else if (run.nadv + 1 == statStep) {
            statBool = true;
        }
        if (exitThisStep) break;
        if (p.endMethod == FIXED_STEP_COUNT) {
            if (run.nadv + 1 == p.stepEnd) exitThisStep = true;
        } else if (run.time + run.dt >= p.tEnd) {
            exitThisStep = true;
            run.flush();          // the last step uses the adjusted dt
            run.dt = p.tEnd - run.time;
        }
    }
    run.flush();
    CHECK(s2d_check_finite(run.h));
    if (!p.checkpoint.empty()) CHECK(s2d_checkpoint_write(run.h, p.checkpoint.c_str(), run.nadv, run.time));
    s2d_destroy(run.h);
    return 0;
}
