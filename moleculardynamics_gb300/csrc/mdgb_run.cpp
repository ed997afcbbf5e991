// mdgb_run: the cpumd program (cpu/cpumd/Main.cpp + Host.cpp:hostMain) with
// the step loop on the GPU engine.
//
// Same command line (one optional configuration file, default "default.cfg",
// common/Loader.cpp:14-29), same inputs (the Input text file, 7 numbers per
// atom, common/Loader.cpp:125-155) and same outputs: the Output text file
// (Loader.cpp:88-120) and the Filename(vxcm-V).dat/.txt results pair
// (common/Results.cpp:120-229), for every vxcm value of the sweep
// (cpu/cpumd/Host.cpp:75).  Errors print a message and exit with
// EXIT_FAILURE, as the reference does.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/mdgb.h"

static void print_record(const md_thermo& r) {
  // common/DebugCalculations.cpp:34-40
  std::cout << "t=" << r.time << "\tT=" << r.temperature << "\tE=" << r.e << "\tEK=" << r.ek
            << "\tEU=" << r.eu << std::endl;
}

static void die(const std::string& msg) {
  std::cerr << "Error: " << msg << std::endl;
  exit(EXIT_FAILURE);
}

int main(int argc, char** argv) {
  std::string cfgfile = "default.cfg";
  if (argc == 2)
    cfgfile = argv[1];
  else if (argc > 2) {
    std::cerr << "usage: mdgb_run [configuration-file].\n";
    return EXIT_FAILURE;
  }
  md_config cfg;
  char strs[2048];
  double extra[6];
  char err[512] = {0};
  if (md_read_config(cfgfile.c_str(), &cfg, strs, extra, err, sizeof(err)) != MD_OK) {
    std::cerr << err << std::endl;
    return EXIT_FAILURE;
  }
  const std::string input = strs, output = strs + 512, filename = strs + 1024,
                    animfile = strs + 1536;
  const int animts = (int)extra[5];
  std::cout << "Molecular::Dynamics\n";
  md_ctx* ctx = nullptr;
  md_status s = md_create(&cfg, &ctx);
  if (s != MD_OK) die(std::string("engine: ") + md_status_string(s));
  // animation frames while animts > -1 (cpu/cpumd/Host.cpp:126,188,212)
  if (animts > -1) {
    const int frames = animts > 0 ? cfg.timesteps / animts + 2 : 2;
    if ((s = md_set_animation(ctx, animts, frames)) != MD_OK) die(md_last_error(ctx));
  }
  const int n = cfg.n_lj + cfg.n_mb;
  std::vector<double> pos(4 * (size_t)n), vel(3 * (size_t)n);
  const float vfrom = (float)extra[1], vto = (float)extra[2], vstep = (float)extra[3];
  for (float vxcm = vfrom; vxcm <= vto; vxcm += vstep) {
    std::ifstream in(input.c_str(), std::ifstream::in);
    if (!in.good()) die("Error opening input file.");
    for (int i = 0; i < n; i++) {
      for (int k = 0; k < 4; k++) in >> pos[4 * (size_t)i + k];
      for (int k = 0; k < 3; k++) in >> vel[3 * (size_t)i + k];
      if (!in.good()) die("Error reading from input file.");
    }
    if ((s = md_upload(ctx, pos.data(), vel.data())) != MD_OK) die(md_last_error(ctx));
    std::cout << std::fixed << std::setprecision(6);
    std::cout.setf(std::ios::fixed, std::ios::floatfield);
    std::cout << "Before Simulation [VXCM = " << vxcm << "]:" << std::endl;
    if ((s = md_begin(ctx, vxcm)) != MD_OK) die(md_last_error(ctx));
    auto t0 = std::chrono::steady_clock::now();
    if ((s = md_step(ctx, cfg.timesteps)) != MD_OK) die(md_last_error(ctx));
    auto t1 = std::chrono::steady_clock::now();
    float elapsed = (float)std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count();
    std::vector<md_thermo> recs(md_record_count(ctx) + 1);
    md_get_records(ctx, recs.data(), (int)recs.size() - 1);
    if (!recs.empty() && recs.size() > 1) print_record(recs[0]);
    std::cout << std::endl;
    md_thermo fin;
    if ((s = md_thermo_now(ctx, &fin)) != MD_OK) die(md_last_error(ctx));
    recs.back() = fin;
    std::cout << "\nAfter Simulation [VXCM = " << vxcm << "]:" << std::endl;
    print_record(fin);
    std::cout << "\nTime took: " << elapsed << "ms" << std::endl << std::endl;
    if ((s = md_download(ctx, pos.data(), vel.data())) != MD_OK) die(md_last_error(ctx));
    std::ofstream out(output.c_str(), std::ofstream::out | std::ofstream::trunc);
    if (!out.good()) die("Error opening output file.");
    out << std::scientific;
    for (int i = 0; i < n; i++) {
      for (int k = 0; k < 4; k++) out << pos[4 * (size_t)i + k] << " ";
      for (int k = 0; k < 3; k++) out << vel[3 * (size_t)i + k] << " ";
      if (!out.good()) die("Error writing to output file file.");
    }
    out.close();
    // the many-body pair list of the .txt, on the device
    int npairs = 0;
    if ((s = md_tail_pairs(ctx, nullptr, 0, &npairs)) != MD_OK) die(md_last_error(ctx));
    std::vector<int> pairs(2 * (size_t)npairs);
    if (npairs > 0 && (s = md_tail_pairs(ctx, pairs.data(), npairs, &npairs)) != MD_OK)
      die(md_last_error(ctx));
    if (md_write_results_pairs(filename.c_str(), &cfg, vxcm, elapsed, recs.data(),
                               (int)recs.size(), pairs.data(), npairs) != MD_OK)
      die("Error writing to result file.");
    if (animts > -1 && md_write_animation(ctx, animfile.c_str(), vxcm) != MD_OK)
      die(md_last_error(ctx));
    if (!(vstep > 0)) break;  // the reference loops forever on a zero step
  }
  md_destroy(ctx);
  return EXIT_SUCCESS;
}
