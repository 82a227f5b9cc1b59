// md_run.cpp -- drop-in executable for MD_Sim_Wolfschwenger's `main`
// (src/simulation.cpp:24-31): InitSimulation then RunSimulation, with the
// time step on the GPU through the library's C ABI (include/md_gb300.h).
//
// Same inputs and outputs as the reference program: the keys of
// configuration.ini (read from ../configuration.ini unless a path is given,
// src/configuration.cpp:6), and in the working directory (or --out DIR)
// data.txt, coords.txt (a frame whenever floor(tInt / tEnd * npCoords)
// reaches the next count, plus the final frame), dtMean.txt, Pxy/Pxz/Pyz.txt,
// MSDx/MSDy/MSDz.txt, mz.txt and t.txt, written with the reference's text
// format (src/postprocessing.cpp, src/simulation.cpp:466-537).
//
// Time stepping: the configuration's SOLVER (0 Heun-Euler, 1
// Bogacki-Shampine, 2 Dormand-Prince) with the reference's step control
// (absTol, deltaTmin, deltaTmax), as the reference runs; --fixed-dt instead
// takes every step with deltaTinit (Heun, every step accepted), the mode of
// the benchmark configurations.
//
// Differences, stated on stdout when they apply:
//   * thermal noise comes from the counter-based Philox generator (or is off,
//     per the [gb300] noise key), not EigenRand's Mersenne Twister;
//   * READ_FROM_FILE reads the last frame of coords_final.txt in the layout
//     WriteCoords2TXT writes (x y z | m | n | label); the reference reads the
//     moments and axes from columns 6-11 of that file, which its own writer
//     does not produce (src/simulation.cpp:375-381 vs
//     src/postprocessing.cpp:84-97).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/md_gb300.h"

namespace {

struct Opts {
  std::string ini = "../configuration.ini";
  std::string out;           // output directory ("" = working directory)
  int precision = -1;        // -1: the configuration's [gb300] precision key
  int autotune = 0;          // candidate cut-offs timed on the device (0: error model + cost model)
  int device = 0;
  int64_t chunk = 100000;    // steps between record read-backs
  bool quiet = false;
  bool fixed_dt = false;     // every step with deltaTinit (Heun)
  std::string resume;        // checkpoint to continue from (md_checkpoint_load)
  std::string checkpoint;    // checkpoint written at the end (md_checkpoint_save)
};

void usage() {
  std::printf(
      "usage: md_run [configuration.ini] [--out DIR] [--precision mixed|fp64] [--autotune K]\n"
      "              [--device D] [--chunk STEPS] [--fixed-dt] [--resume FILE] [--checkpoint FILE]\n"
      "              [--quiet]\n"
      "Runs MD_Sim_Wolfschwenger's simulation (InitSimulation + RunSimulation) with the time step on\n"
      "the GPU; the configuration defaults to ../configuration.ini like the reference.\n");
}

[[noreturn]] void die(md_ctx* ctx, int st, const char* what) {
  char buf[1024] = {0};
  md_last_error(ctx, buf, sizeof buf);
  std::fprintf(stderr, "md_run: %s failed: %s (%s)\n", what, md_strerror(st), buf);
  std::exit(1);
}

#define CALL(ctx, expr)                   \
  do {                                    \
    const int st_ = (expr);               \
    if (st_ != MD_OK) die(ctx, st_, #expr); \
  } while (0)

std::string path_in(const Opts& o, const char* name) {
  if (o.out.empty()) return name;
  return o.out + (o.out.back() == '/' ? "" : "/") + name;
}

// Last frame of a coords file written by WriteCoords2TXT: rows of 10
// numbers, frames separated by empty lines.
bool read_last_frame(const std::string& path, int64_t n, std::vector<double>* pos, std::vector<double>* mm,
                     std::vector<double>* ea) {
  std::ifstream f(path);
  if (!f) return false;
  std::vector<std::vector<double>> frame, last;
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::vector<double> row;
    double v;
    while (ss >> v) row.push_back(v);
    if (row.empty()) {
      if (!frame.empty()) last.swap(frame);
      frame.clear();
      continue;
    }
    if (row.size() < 9) return false;
    frame.push_back(row);
  }
  if (!frame.empty()) last.swap(frame);
  if ((int64_t)last.size() != n) return false;
  for (int64_t i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) {
      (*pos)[(size_t)(i + c * n)] = last[(size_t)i][(size_t)c];
      (*mm)[(size_t)(i + c * n)] = last[(size_t)i][(size_t)(3 + c)];
      (*ea)[(size_t)(i + c * n)] = last[(size_t)i][(size_t)(6 + c)];
    }
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  Opts o;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    auto next = [&](const char* what) -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "md_run: %s needs a value\n", what);
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "-h" || a == "--help") {
      usage();
      return 0;
    } else if (a == "--out") {
      o.out = next("--out");
    } else if (a == "--precision") {
      const std::string p = next("--precision");
      if (p == "mixed") o.precision = MD_PREC_MIXED;
      else if (p == "fp64") o.precision = MD_PREC_FP64;
      else { std::fprintf(stderr, "md_run: precision must be mixed or fp64\n"); return 2; }
    } else if (a == "--autotune") {
      o.autotune = std::atoi(next("--autotune"));
    } else if (a == "--device") {
      o.device = std::atoi(next("--device"));
    } else if (a == "--chunk") {
      o.chunk = std::max<int64_t>(1, std::atoll(next("--chunk")));
    } else if (a == "--quiet") {
      o.quiet = true;
    } else if (a == "--fixed-dt") {
      o.fixed_dt = true;
    } else if (a == "--resume") {
      o.resume = next("--resume");
    } else if (a == "--checkpoint") {
      o.checkpoint = next("--checkpoint");
    } else if (!a.empty() && a[0] == '-') {
      std::fprintf(stderr, "md_run: unknown option %s\n", a.c_str());
      usage();
      return 2;
    } else {
      o.ini = a;
    }
  }

  // ----------------------------------------------------- InitSimulation
  md_config cfg;
  CALL(nullptr, md_config_load_ini(o.ini.c_str(), &cfg));
  const int prec = o.precision >= 0 ? o.precision : (int)cfg.precision;
  const int64_t n = md_config_numb_part(&cfg);
  if (!o.fixed_dt && (cfg.SOLVER < 0 || cfg.SOLVER > 2)) {
    std::fprintf(stderr, "md_run: SOLVER must be 0, 1 or 2\n");
    return 1;
  }
  if (o.fixed_dt)
    std::printf("note: fixed step deltaTinit = %g s (Heun, every step accepted)\n", cfg.deltaTinit);
  std::vector<double> rMag((size_t)n), rHydr((size_t)n), pos(3 * (size_t)n), mm(3 * (size_t)n), ea(3 * (size_t)n);
  double lBox = 0;
  CALL(nullptr, md_init_system(&cfg, n, (uint64_t)cfg.seed, rMag.data(), rHydr.data(), pos.data(), mm.data(),
                               ea.data(), &lBox));
  if (cfg.READ_FROM_FILE) {
    const std::string src = path_in(o, "coords_final.txt");
    if (!read_last_frame(src, n, &pos, &mm, &ea)) {
      std::fprintf(stderr, "md_run: READ_FROM_FILE: %s does not hold a frame of %lld particles\n", src.c_str(),
                   (long long)n);
      return 1;
    }
  }
  CALL(nullptr, md_select_device(o.device));
  md_ctx* ctx = nullptr;
  CALL(nullptr, md_ctx_create(&cfg, n, prec, &ctx));
  CALL(ctx, md_set_particles(ctx, rMag.data(), rHydr.data()));
  CALL(ctx, md_set_box(ctx, lBox));
  CALL(ctx, md_state_upload(ctx, pos.data(), mm.data(), ea.data(), 1));
  double alpha = 0, rc = 0, errF = 0, errT = 0, ms = 0;
  int64_t kc = 0;
  if (o.autotune > 0) {
    CALL(ctx, md_autotune_ewald(ctx, o.autotune, &alpha, &rc, &kc, &ms));
  } else {
    CALL(ctx, md_ewald_params(ctx, -1.0, &alpha, &rc, &kc, &errF, &errT));
    CALL(ctx, md_set_ewald(ctx, alpha, rc, kc));
  }
  CALL(ctx, md_ewald_params(ctx, rc, &alpha, &rc, &kc, &errF, &errT));
  std::printf("particles: %lld, box length: %g m, precision: %s\n", (long long)n, lBox,
              prec == MD_PREC_FP64 ? "fp64" : "mixed");
  std::printf("Ewald: alpha = %g 1/m, rc = %g m (%.4g L), kc = %lld; predicted force error %.3g, torque error "
              "%.3g (relative to contact)\n",
              alpha, rc, rc / lBox, (long long)kc, errF, errT);
  CALL(ctx, md_set_noise(ctx, (int)cfg.noise, (uint64_t)cfg.seed));
  double t_start = 0;  // time of the first step (later than 0 when resuming)
  if (!o.resume.empty()) {
    // continue a run: radii, box, Ewald parameters, state, time and noise
    // counter from the checkpoint; the loop below runs on until tEnd
    CALL(ctx, md_checkpoint_load(ctx, o.resume.c_str()));
    CALL(ctx, md_get_box(ctx, &lBox));
    int64_t s0 = 0;
    CALL(ctx, md_get_time(ctx, &t_start, &s0));
    std::printf("resumed from %s at t = %g s (step %lld), with its Ewald parameters\n", o.resume.c_str(), t_start,
                (long long)s0);
  }
  CALL(nullptr, md_write_data_txt(path_in(o, "data.txt").c_str(), &cfg, n, rMag.data(), rHydr.data(), lBox));

  // ------------------------------------------------------ RunSimulation
  // The frame test sits at the top of the loop body and its frame is written
  // after the step with the step's start time (src/simulation.cpp:466-520).
  const double tEnd = cfg.tEnd;
  const std::string coords = path_in(o, "coords.txt");
  std::vector<double> rec;
  auto pull_records = [&]() {
    int64_t nr = 0;
    CALL(ctx, md_num_records(ctx, &nr));
    const size_t at = rec.size();
    rec.resize(at + 8 * (size_t)nr);
    CALL(ctx, md_records(ctx, 0, nr, rec.data() + at));
    CALL(ctx, md_clear_records(ctx));
  };
  auto write_frame = [&](double label, int64_t count) {
    CALL(ctx, md_state_download(ctx, pos.data(), mm.data(), ea.data()));
    CALL(nullptr, md_write_coords_txt(coords.c_str(), n, pos.data(), mm.data(), ea.data(), label));
    if (!o.quiet)
      std::printf("actual time: %gs\nsimulation progress: %g%%\n", label, (double)count / cfg.npCoords * 100.0);
  };
  int64_t steps = 0;
  double tInt = t_start;
  // frames already written before a resumed run's start
  const int64_t count0 = t_start > 0 ? (int64_t)std::floor(t_start / tEnd * cfg.npCoords) + 1 : 0;
  if (o.fixed_dt) {
    // time points and frames with the reference's own double arithmetic
    const double dt = cfg.deltaTinit;
    struct Frame {
      int64_t step;
      double t;
    };
    std::vector<Frame> frames;
    {
      int64_t count = count0;
      while (tInt <= tEnd) {
        if (std::floor(tInt / tEnd * cfg.npCoords) == (double)count) {
          frames.push_back({steps, tInt});
          count++;
        }
        tInt += dt;
        steps++;
      }
    }
    rec.reserve(8 * (size_t)steps);
    int64_t done = 0;
    auto advance = [&](int64_t upto) {  // runs steps [done, upto)
      while (done < upto) {
        const int64_t k = std::min(o.chunk, upto - done);
        CALL(ctx, md_step(ctx, k, dt, nullptr));
        pull_records();
        done += k;
      }
    };
    for (size_t f = 0; f < frames.size(); f++) {
      advance(frames[f].step + 1);
      write_frame(frames[f].t, (int64_t)f);
    }
    advance(steps);
  } else {
    // adaptive: one accepted step at a time (the next time point is known
    // only after the step control has run)
    double dt = cfg.deltaTinit;
    int64_t count = count0;
    while (tInt <= tEnd) {
      const bool frame = std::floor(tInt / tEnd * cfg.npCoords) == (double)count;
      int64_t k = 0;
      CALL(ctx, md_step_adaptive(ctx, 1, tEnd, &dt, nullptr, &k));
      if (k != 1) break;
      if (frame) write_frame(tInt, count++);
      int64_t sdev = 0;
      CALL(ctx, md_get_time(ctx, &tInt, &sdev));
      steps++;
      if (steps % o.chunk == 0) pull_records();
    }
    pull_records();
  }
  double tDev = 0;
  int64_t sDev = 0;
  CALL(ctx, md_get_time(ctx, &tDev, &sDev));
  std::printf("simulation progress: 100%%\n%lld timesteps needed\n", (long long)steps);
  CALL(ctx, md_state_download(ctx, pos.data(), mm.data(), ea.data()));
  CALL(nullptr, md_write_coords_txt(coords.c_str(), n, pos.data(), mm.data(), ea.data(), tInt));
  CALL(nullptr, md_export_records_txt(o.out.c_str(), rec.data(), (int64_t)(rec.size() / 8), tInt, steps));
  if (tDev != tInt || sDev != steps)
    std::printf("note: device time %.17g after %lld steps, host %.17g after %lld\n", tDev, (long long)sDev, tInt,
                (long long)steps);
  if (!o.checkpoint.empty()) CALL(ctx, md_checkpoint_save(ctx, o.checkpoint.c_str()));
  md_ctx_destroy(ctx);
  std::printf("simulation ended successfully\n");
  return 0;
}
