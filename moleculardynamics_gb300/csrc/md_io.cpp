// Configuration and results files of the reference, on the host.
//
// md_read_config follows common/ConfigParser.cpp:22-156 and
// common/Loader.cpp:34-83: key=value lines read by the rules R1-R6 below,
// numbers read with istream >> (bools as 0/1), and the 25 keys of
// Loader.cpp:49-82 mandatory.
// md_write_results writes the .dat/.txt pair of common/Results.cpp:120-229
// and the pair list of common/Results.cpp:88-118.
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mdgb.h"

namespace {

struct Parsed {
  std::unordered_map<std::string, std::string> kv;
  std::string err;
};

std::string upper(std::string s) {
  for (auto& ch : s) ch = (char)toupper((unsigned char)ch);
  return s;
}

// The reference's reading rules (common/ConfigParser.cpp:22-98), one by one:
//  R1 lines as std::getline splits the file: a last line without '\n'
//     counts, the empty segment after a final '\n' does not;
//  R2 empty lines and lines that begin with "//" are skipped;
//  R3 comments are cut at the LAST "//" again and again until none is left,
//     so "a///b" keeps "a/";
//  R4 the key is the text before the first '=', upper-cased and not
//     trimmed; a line without '=' or with an empty key is an error that
//     names how many key lines were read before it;
//  R5 blanks (space, tab) are cut from the end of the value, unless the
//     value is all blanks or its only non-blank character is its first;
//  R6 the first line of a key wins.
namespace rules {
bool skipped(const std::string& l) { return l.empty() || l.compare(0, 2, "//") == 0; }  // R2
std::string uncomment(std::string l) {                                                   // R3
  for (size_t at; (at = l.rfind("//")) != std::string::npos;) l.erase(at);
  return l;
}
std::string trim_value(const std::string& v) {  // R5
  const size_t last = v.find_last_not_of(" \t");
  return last == std::string::npos || last == 0 ? v : v.substr(0, last + 1);
}
}  // namespace rules

bool parse_file(const char* path, Parsed& p) {
  std::ifstream in(path);
  if (!in) {
    p.err = "Error opening configuration file.";
    return false;
  }
  int keys = 0;
  for (std::string raw; std::getline(in, raw);) {  // R1
    if (rules::skipped(raw)) continue;
    const std::string line = rules::uncomment(raw);
    const size_t eq = line.find('=');
    if (eq == std::string::npos || eq == 0) {  // R4
      p.err = "Error in configuration file!\nLine: " + std::to_string(keys);
      return false;
    }
    p.kv.emplace(upper(line.substr(0, eq)), rules::trim_value(line.substr(eq + 1)));  // R6
    keys++;
  }
  if (!in.eof()) {  // a read that failed before the end of the file
    p.err = "Unable to read line from configuration file.";
    return false;
  }
  return true;
}

template <typename T>
bool from_string(T& t, const std::string& s) {
  std::istringstream iss(s);
  return !(iss >> std::dec >> t).fail();
}

bool get_str(Parsed& p, const char* key, std::string& v) {
  auto it = p.kv.find(upper(key));
  if (it == p.kv.end()) return false;
  v = it->second;
  return true;
}
template <typename T>
bool get_num(Parsed& p, const char* key, T& v) {
  auto it = p.kv.find(upper(key));
  if (it == p.kv.end()) return false;
  return from_string<T>(v, it->second);
}
bool get_bool(Parsed& p, const char* key, int& v) {
  bool b = false;
  bool ok = get_num<bool>(p, key, b);
  v = b ? 1 : 0;
  return ok;
}

void put(char* dst, const std::string& s) {
  strncpy(dst, s.c_str(), 511);
  dst[511] = 0;
}

}  // namespace

extern "C" md_status md_read_config(const char* path, md_config* cfg, char* strings,
                                    double* extra, char* err, int err_len) {
  auto set_err = [&](const std::string& m) {
    if (err && err_len > 0) {
      strncpy(err, m.c_str(), (size_t)err_len - 1);
      err[err_len - 1] = 0;
    }
  };
  if (!path || !cfg) return MD_BAD_ARGUMENT;
  Parsed p;
  if (!parse_file(path, p)) {
    set_err(p.err);
    return MD_BAD_CONFIG;
  }
  md_config c;
  memset(&c, 0, sizeof(c));
  int cudablocks = 0, animts = 0, usecuda = 0, ljbpp = 0, mbbpp = 0, debug = 0, fallback = 0;
  float temp = 0, vfrom = 0, vto = 0, vstep = 0;
  std::string in, out, fname, anim;
  bool v = true;
  // common/Loader.cpp:49-76 (same order)
  v &= get_num(p, "Lennard Jones Particles", c.n_lj);
  v &= get_num(p, "Timesteps", c.timesteps);
  v &= get_num(p, "DT", c.dt);
  v &= get_num(p, "Temperature", temp);
  v &= get_num(p, "LennardJonesRS", c.lj_rs);
  v &= get_num(p, "LennardJonesRCUT", c.lj_rcut);
  v &= get_num(p, "ManyBodyRS", c.mb_rs);
  v &= get_num(p, "ManyBodyRCUT", c.mb_rcut);
  v &= get_str(p, "Input", in);
  v &= get_str(p, "Output", out);
  v &= get_str(p, "Filename", fname);
  v &= get_num(p, "CUDA Blocks", cudablocks);
  v &= get_bool(p, "Use Cuda", usecuda);
  v &= get_num(p, "OutputTimesteps", c.output_timesteps);
  v &= get_bool(p, "Debug", debug);
  v &= get_bool(p, "Fallback", fallback);
  v &= get_bool(p, "UseLennardJones", c.use_lj);
  v &= get_bool(p, "UseManyBody", c.use_mb);
  v &= get_bool(p, "LennardJonesBPP", ljbpp);
  v &= get_bool(p, "ManyBodyBPP", mbbpp);
  v &= get_num(p, "VXCMFROM", vfrom);
  v &= get_num(p, "VXCMTO", vto);
  v &= get_num(p, "VXCMSTEP", vstep);
  v &= get_num(p, "EnergyLoss", c.energy_loss);
  v &= get_num(p, "Many Body Particles", c.n_mb);
  v &= get_num(p, "AnimationTimesteps", animts);
  v &= get_str(p, "AnimationData", anim);
  if (!v) {
    set_err("Unable to read configuration file!");
    return MD_BAD_CONFIG;
  }
  // extension keys (absent = the reference's behaviour)
  std::string sv;
  if (get_str(p, "Periodic", sv) && !get_bool(p, "Periodic", c.periodic)) {
    set_err("bad value for Periodic");
    return MD_BAD_CONFIG;
  }
  if (get_str(p, "Box", sv) && !get_num(p, "Box", c.box)) {
    set_err("bad value for Box");
    return MD_BAD_CONFIG;
  }
  if (get_str(p, "Precision", sv)) {
    std::string u = upper(sv);
    if (u.rfind("MIXED", 0) == 0 || u.rfind("FP32", 0) == 0)
      c.precision = MD_PREC_MIXED;
    else if (u.rfind("FP64", 0) == 0 || u.rfind("PLAIN", 0) == 0)
      c.precision = MD_PREC_FP64;
    else {
      set_err("bad value for Precision (FP64 or MIXED)");
      return MD_BAD_CONFIG;
    }
  }
  if (get_str(p, "Species", sv)) {
    std::string u = upper(sv);
    if (u.rfind("ARGON", 0) == 0)
      c.species = MD_SPECIES_ARGON;
    else if (u.rfind("NEON", 0) == 0 || u.rfind("REFERENCE", 0) == 0)
      c.species = MD_SPECIES_NEON;
    else {
      set_err("bad value for Species (NEON or ARGON)");
      return MD_BAD_CONFIG;
    }
  }
  if (get_str(p, "Device", sv) && !get_num(p, "Device", c.device)) {
    set_err("bad value for Device");
    return MD_BAD_CONFIG;
  }
  if (get_str(p, "ReferenceEnergy", sv) &&
      (!get_num(p, "ReferenceEnergy", c.reference_energy) || c.reference_energy < 0 ||
       c.reference_energy > 2)) {
    set_err("bad value for ReferenceEnergy (0, 1 or 2)");
    return MD_BAD_CONFIG;
  }
  if (get_str(p, "LJKernel", sv)) {
    std::string u = upper(sv);
    if (u.rfind("AUTO", 0) == 0)
      c.lj_kernel = MD_LJ_AUTO;
    else if (u.rfind("ROWS", 0) == 0)
      c.lj_kernel = MD_LJ_ROWS;
    else if (u.rfind("CLUSTER", 0) == 0)
      c.lj_kernel = MD_LJ_CLUSTER;
    else {
      set_err("bad value for LJKernel (AUTO, ROWS or CLUSTER)");
      return MD_BAD_CONFIG;
    }
  }
  *cfg = c;
  if (strings) {
    put(strings, in);
    put(strings + 512, out);
    put(strings + 1024, fname);
    put(strings + 1536, anim);
  }
  if (extra) {
    extra[0] = temp;
    extra[1] = vfrom;
    extra[2] = vto;
    extra[3] = vstep;
    extra[4] = cudablocks;
    extra[5] = animts;
  }
  return MD_OK;
}

namespace {

// common/Results.cpp:88-118 tailResults: the text of the pair list
std::string tail_text(const int* pairs, int npairs) {
  std::stringstream ssPairs, tail;
  tail << "ManyBody Pairs:\n";
  for (int k = 0; k < npairs; k++) ssPairs << "[" << pairs[2 * k] << ", " << pairs[2 * k + 1] << "] ";
  tail << "Amount: " << npairs << "\n" << ssPairs.str();
  return tail.str();
}

// common/Results.cpp:120-229 writeResults with the tail text given
md_status write_results(const char* filename, const md_config* cfg, float vxcm, float elapsed,
                        const md_thermo* recs, int nrec, const std::string& tail_str) {
  std::stringstream rf, lf;
  rf << filename << "(vxcm-" << vxcm << ").dat";
  lf << filename << "(vxcm-" << vxcm << ").txt";
  std::ofstream result(rf.str().c_str(), std::fstream::binary | std::fstream::out | std::fstream::trunc);
  if (result.fail()) return MD_BAD_ARGUMENT;
  std::ofstream log(lf.str().c_str(), std::ofstream::out | std::ofstream::trunc);
  if (log.fail()) return MD_BAD_ARGUMENT;
  log << std::fixed << std::setprecision(6);
  log.setf(std::ios::fixed, std::ios::floatfield);
  log << "Number Of Particles = " << cfg->n_lj + cfg->n_mb << ", Timesteps = " << cfg->timesteps
      << "\n";
  log << "DT = " << cfg->dt;
  if (cfg->use_lj)
    log << ", LennardJonesRS = " << cfg->lj_rs << ", LennardJonesRCUT = " << cfg->lj_rcut;
  if (cfg->use_mb)
    log << ", ManyBodyRS = " << cfg->mb_rs << ", ManyBodyRCUT = " << cfg->mb_rcut;
  log << "\n\n";
  log << "\nVXCM [" << vxcm << "]: Time took: " << elapsed << " ms\n\n";
  log << "t\t\tT\t\tE\t\tEK\t\tEU\t\tR.x\t\tR.y\t\tR.z\t\tp.x\t\tp.y\t\tp.z\n";
  int nop = cfg->n_lj + cfg->n_mb;
  result.write((const char*)&nop, sizeof(int));
  result.write((const char*)&cfg->timesteps, sizeof(int));
  result.write((const char*)&cfg->dt, sizeof(float));
  unsigned char b = cfg->use_lj ? 0xFF : 0x00;
  result.write((const char*)&b, 1);
  if (cfg->use_lj) {
    result.write((const char*)&cfg->lj_rs, sizeof(float));
    result.write((const char*)&cfg->lj_rcut, sizeof(float));
  }
  b = cfg->use_mb ? 0xFF : 0x00;
  result.write((const char*)&b, 1);
  if (cfg->use_mb) {
    result.write((const char*)&cfg->mb_rs, sizeof(float));
    result.write((const char*)&cfg->mb_rcut, sizeof(float));
  }
  result.write((const char*)&vxcm, sizeof(float));
  for (int k = 0; k < nrec; k++) {
    const md_thermo& r = recs[k];
    log << std::endl;
    result.write((const char*)&r, 11 * sizeof(double));  // struct results order
    log << r.time;
    log << std::scientific;
    log << "\t" << r.temperature << "\t" << r.e << "\t" << r.ek << "\t" << r.eu << "\t" << r.com_x
        << "\t" << r.com_y << "\t" << r.com_z << "\t" << r.momentum_x << "\t" << r.momentum_y
        << "\t" << r.momentum_z;
    log << std::fixed;
  }
  log << "\n\n" << tail_str;
  if (result.fail() || log.fail()) return MD_BAD_ARGUMENT;
  return MD_OK;
}

}  // namespace

extern "C" md_status md_write_results(const char* filename, const md_config* cfg, float vxcm,
                                      float elapsed, const md_thermo* recs, int nrec,
                                      const double* pos4) {
  if (!filename || !cfg || (nrec > 0 && !recs)) return MD_BAD_ARGUMENT;
  // common/Results.cpp:88-118 tailResults over the many-body atoms
  std::vector<int> pairs;
  for (int i = 0; pos4 && i < cfg->n_mb; i++)
    for (int j = i + 1; j < cfg->n_mb; j++) {
      if ((int)pos4[4 * i + 3] == (int)pos4[4 * j + 3]) continue;
      double dx = pos4[4 * i] - pos4[4 * j];
      double dy = pos4[4 * i + 1] - pos4[4 * j + 1];
      double dz = pos4[4 * i + 2] - pos4[4 * j + 2];
      double dist = sqrt(dx * dx + dy * dy + dz * dz);
      if (dist < 2 * 1.15f) {
        pairs.push_back(i);
        pairs.push_back(j);
      }
    }
  return write_results(filename, cfg, vxcm, elapsed, recs, nrec,
                       tail_text(pairs.data(), (int)pairs.size() / 2));
}

extern "C" md_status md_write_results_pairs(const char* filename, const md_config* cfg,
                                            float vxcm, float elapsed, const md_thermo* recs,
                                            int nrec, const int* pairs, int npairs) {
  if (!filename || !cfg || (nrec > 0 && !recs) || npairs < 0 || (npairs > 0 && !pairs))
    return MD_BAD_ARGUMENT;
  return write_results(filename, cfg, vxcm, elapsed, recs, nrec, tail_text(pairs, npairs));
}
