// sop_gpu.x -- the reference program's command-line drop-in on the GB300 engine.
//
//   sop_gpu.x <input_file>
//
// Reads the reference's command script (io.cpp:9-89: blank-separated tokens,
// a command and its options ending at a token that holds ';') and executes
// it in order like ex_cmds (sop.cpp:58-72):
//   load bonds|angles|vdw|init <file>   the data files (params.cpp:110-260)
//   set <key> <value>                   parameters with set_params' side
//                                       effects (params.cpp:12-101)
//   run                                 the simulation (sop.cpp:74-198,
//                                       365-471), on the GPU
// and writes what the reference writes every nup steps: a row of ufname
// (default update.out, appended: "istep T kinT e_bnd e_ang_ss e_vdw_rr
// rna_etot Q contct_nat rgsq"), the coordinates (cfname, unccfname) and the
// velocities (vfname), and a frame appended to each trajectory file (binfname,
// uncbinfname; text frames, as record_traj writes them, starting with the
// initial coordinates).  The reference's sequential random stream is not
// reproduced: noise comes from the engine's
// counter-based stream keyed by -100-run.  A vdw file listing fewer non-native
// candidates than all pairs |i-j| > 2 is honoured through exclusions.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_set>
#include <vector>

#include "../../include/sop_gpu.h"

namespace {

struct Command {
  std::string cmd;
  std::vector<std::string> opt;
};

// io.cpp:9-89: tokens split on blanks; a token holding ';' ends a command.
std::vector<Command> read_input(const char* path) {
  std::ifstream in(path);
  if (!in) {
    std::fprintf(stderr, "cannot open %s\n", path);
    std::exit(1);
  }
  std::vector<Command> cmds;
  std::string line;
  bool fresh = true;
  while (std::getline(in, line)) {
    std::stringstream ss(line);
    std::string tok;
    while (std::getline(ss, tok, ' ')) {
      if (tok.empty()) continue;
      const bool ends = tok.find(';') != std::string::npos;
      std::string clean;
      for (char c : tok)
        if (c != ';' && c != '\r' && c != '\t') clean += c;
      if (fresh) {
        cmds.push_back(Command{clean, {}});
        fresh = false;
      } else if (!cmds.empty()) {
        cmds.back().opt.push_back(clean);
      }
      if (ends) fresh = true;
    }
  }
  return cmds;
}

// The parameters the script sets, with set_params' side effects.
struct Settings {
  double T = 0.6, zeta = 5.0e-2, h = 2.5e-3, halfh = 1.25e-3;
  double a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0;
  double boxl = 500.0, ncell = 55.0, lcell = 500.0 / 55.0;
  double nstep = 5.0e7, istep_restart = 0.0;
  int nup = 1000, nnlup = 50, run = 1, sim_type = 1;
  int neighborlist = 0, celllist = 0, restart = 0, rgen_restart = 0;
  std::string ufname = "update.out", cfname = "coord.out", unccfname = "unccoord.out",
              vfname = "veloc.out", rcfname = "restart_c.dat", binfname = "traj.bin",
              uncbinfname = "traj_uncorrected.bin";

  void integ() {  // params.cpp:22-27
    a1 = h * (1.0 - zeta * halfh);
    a2 = h * halfh;
    a3 = (1.0 - h * zeta / 2.0 + (h * zeta) * (h * zeta) / 4.0) / h;
    a4 = halfh * (1.0 - h * zeta / 2.0);
  }
  Settings() {
    integ();
    a5 = h / zeta;  // params.cpp:392
  }
  void set(const std::string& key, const std::string& val) {
    const double v = std::atof(val.c_str());
    if (key == "dynamics") {
      if (val == "underdamped") {
        sim_type = 1;
        h = 2.5e-3;
        halfh = h / 2.0;
        integ();
      } else if (val == "overdamped") {
        sim_type = 2;
        h = 0.02;
        a5 = h / zeta;
      }
    } else if (key == "temp") {
      T = v;
    } else if (key == "nstep") {
      nstep = v;
    } else if (key == "istep_restart") {
      istep_restart = v;
    } else if (key == "nup") {
      nup = std::atoi(val.c_str());
    } else if (key == "run") {
      run = std::atoi(val.c_str());
    } else if (key == "ufname") {
      ufname = val;
    } else if (key == "rcfname") {
      rcfname = val;
    } else if (key == "cfname") {
      cfname = val;
    } else if (key == "unccfname") {
      unccfname = val;
    } else if (key == "vfname") {
      vfname = val;
    } else if (key == "binfname") {
      binfname = val;
    } else if (key == "uncbinfname") {
      uncbinfname = val;
    } else if (key == "cutofftype") {
      if (val == "neighborlist") neighborlist = 1;
      else if (val == "celllist") celllist = 1;
    } else if (key == "nnlup") {
      nnlup = std::atoi(val.c_str());
    } else if (key == "boxl") {
      boxl = v;
    } else if (key == "ncell") {
      ncell = v;
      lcell = boxl / ncell;
    } else if (key == "restart") {
      restart = val == "on";
    } else if (key == "rgen_restart") {
      rgen_restart = val == "on";
    } else if (key == "t_step") {
      h = v;
      halfh = h / 2.0;
      integ();
      a5 = h / zeta;
    } else if (key == "zeta") {
      if (sim_type == 1) h = 2.5e-3;
      else if (sim_type == 2) h = 0.02;
      zeta = v;
      a1 = h * (1.0 - zeta * halfh);
      a3 = (1.0 - h * zeta / 2.0 + (h * zeta) * (h * zeta) / 4.0) / h;
      a4 = halfh * (1.0 - h * zeta / 2.0);
      a5 = h / zeta;
    }
  }
};

struct Topology {
  int nbead = 0;
  std::vector<double> xyz;
  std::vector<int> type, ib, jb, ia, ka, in_, jn, ie, je;
  std::vector<double> r0, rn;
  bool have_vdw = false;
  long long listed_rep = 0;
  std::vector<std::pair<int, int>> rep_pairs;  // listed non-native candidates (i < j)
};

std::vector<std::string> split(const std::string& s) {
  std::vector<std::string> out;
  std::stringstream ss(s);
  std::string t;
  while (ss >> t) out.push_back(t);
  return out;
}

// A data file is refused, with the reason on stderr, when it declares more
// entries than it holds, when an entry has too few fields, or when a bead
// index is not 1..kMaxBeads (the reference reads such files without checks,
// params.cpp:110-260; indices past the loaded chain are refused by the engine).
constexpr long long kMaxBeads = 1LL << 22;

bool bad_entry(const std::string& file, long long k, const char* why) {
  std::fprintf(stderr, "%s: entry %lld: %s\n", file.c_str(), k + 1, why);
  return false;
}

bool bead_index(const std::string& tok, int* out) {
  const long long v = std::atoll(tok.c_str());
  if (v < 1 || v > kMaxBeads) return false;
  *out = (int)(v - 1);
  return true;
}

bool load(const Command& c, Topology& top) {
  if (c.opt.size() < 2) return false;
  const std::string& file = c.opt[1];
  std::ifstream in(file);
  if (!in) {
    std::fprintf(stderr, "cannot open %s\n", file.c_str());
    return false;
  }
  std::string line;
  std::getline(in, line);
  const std::vector<std::string> head = split(line);
  const std::string& what = c.opt[0];
  if (what == "bonds" && head.size() >= 2) {  // params.cpp:126-144
    const long long n = std::atoll(head[1].c_str());
    for (long long k = 0; k < n; k++) {
      if (!std::getline(in, line)) return bad_entry(file, k, "missing (the header declares more)");
      const auto t = split(line);
      int i, j;
      if (t.size() < 3) return bad_entry(file, k, "fewer than 3 fields");
      if (!bead_index(t[0], &i) || !bead_index(t[1], &j)) return bad_entry(file, k, "bead index out of range");
      top.ib.push_back(i);
      top.jb.push_back(j);
      top.r0.push_back(std::atof(t[2].c_str()));
    }
  } else if (what == "angles" && head.size() >= 2) {  // params.cpp:145-165
    const long long n = std::atoll(head[1].c_str());
    for (long long k = 0; k < n; k++) {
      if (!std::getline(in, line)) return bad_entry(file, k, "missing (the header declares more)");
      const auto t = split(line);
      int i, j, m;
      if (t.size() < 4) return bad_entry(file, k, "fewer than 4 fields");
      if (!bead_index(t[0], &i) || !bead_index(t[1], &j) || !bead_index(t[2], &m))
        return bad_entry(file, k, "bead index out of range");
      top.ia.push_back(i);
      top.ka.push_back(m);
    }
  } else if (what == "vdw" && head.size() >= 4) {  // params.cpp:166-234
    const long long n = std::atoll(head[1].c_str()) + std::atoll(head[3].c_str());
    top.have_vdw = true;
    for (long long k = 0; k < n; k++) {
      if (!std::getline(in, line)) return bad_entry(file, k, "missing (the header declares more)");
      const auto t = split(line);
      int i, j;
      if (t.size() < 5) return bad_entry(file, k, "fewer than 5 fields");
      if (!bead_index(t[0], &i) || !bead_index(t[1], &j)) return bad_entry(file, k, "bead index out of range");
      const double r = std::atof(t[2].c_str());
      const int ti = std::atoi(t[3].c_str()), tj = std::atoi(t[4].c_str());
      if ((int)top.type.size() < std::max(i, j) + 1) top.type.resize(std::max(i, j) + 1, 1);
      top.type[i] = ti;
      top.type[j] = tj;
      // every listed pair goes to the engine, which keeps r < rcut_nat as
      // natives (params.cpp:197); the rest are the listed non-native candidates
      top.in_.push_back(std::min(i, j));
      top.jn.push_back(std::max(i, j));
      top.rn.push_back(r);
      top.rep_pairs.push_back({std::min(i, j), std::max(i, j)});
    }
  } else if (what == "init" && head.size() >= 2) {  // params.cpp:235-258
    const long long n = std::atoll(head[1].c_str());
    if (n < 1 || n > kMaxBeads) {
      std::fprintf(stderr, "%s: bead count %lld out of range\n", file.c_str(), n);
      return false;
    }
    top.nbead = (int)n;
    top.xyz.assign(3 * (size_t)top.nbead, 0.0);
    for (long long k = 0; k < n; k++) {
      if (!std::getline(in, line)) return bad_entry(file, k, "missing (the header declares more)");
      const auto t = split(line);
      if (t.size() < 4) return bad_entry(file, k, "fewer than 4 fields");
      for (int q = 0; q < 3; q++) top.xyz[3 * k + q] = std::atof(t[1 + q].c_str());
    }
  } else {
    std::fprintf(stderr, "%s: unknown data kind '%s' or header\n", file.c_str(), what.c_str());
    return false;
  }
  return true;
}

// Pairs of the implicit candidate set (|i-j| > 2) the vdw file does not list
// must not interact: they become exclusions.
void exclusions(Topology& top) {
  const int n = top.nbead;
  std::unordered_set<unsigned long long> listed;
  listed.reserve(top.rep_pairs.size() * 2);
  for (auto& p : top.rep_pairs) listed.insert((unsigned long long)p.first * n + p.second);
  const long long implicit = n > 3 ? (long long)(n - 3) * (n - 2) / 2 : 0;
  if ((long long)listed.size() >= implicit) return;  // every candidate listed
  for (int i = 0; i < n; i++)
    for (int j = i + 3; j < n; j++)
      if (!listed.count((unsigned long long)i * n + j)) {
        top.ie.push_back(i);
        top.je.push_back(j);
      }
}

void write_coords(const std::string& fname, const std::vector<double>& x, int n) {
  FILE* f = std::fopen(fname.c_str(), "w");
  if (!f) return;
  for (int i = 0; i < n; i++) std::fprintf(f, "%d %f %f %f\n", i + 1, x[3 * i], x[3 * i + 1], x[3 * i + 2]);
  std::fclose(f);
}

// record_traj (io.cpp:280-303): one "%f %f %f" line per bead appended to the
// file; despite the ".bin" default names the frames are text.
void append_frame(const std::string& fname, const std::vector<double>& x, int n) {
  FILE* f = std::fopen(fname.c_str(), "a");
  if (!f) return;
  for (int i = 0; i < n; i++) std::fprintf(f, "%f %f %f\n", x[3 * i], x[3 * i + 1], x[3 * i + 2]);
  std::fclose(f);
}

// n coordinate lines "index x y z" (io.cpp's coordinate format); false when
// the file is missing or holds fewer.
bool read_coords(const std::string& fname, std::vector<double>& x, int n) {
  std::ifstream in(fname);
  if (!in) return false;
  std::string line;
  for (int i = 0; i < n; i++) {
    if (!std::getline(in, line)) return false;
    const auto t = split(line);
    if (t.size() < 4) return false;
    for (int q = 0; q < 3; q++) x[3 * i + q] = std::atof(t[1 + q].c_str());
  }
  return true;
}

int check(int rc, const char* what) {
  if (rc != SOP_OK) {
    std::fprintf(stderr, "%s failed: %s (%d)\n", what, sop_status_string(rc), rc);
    std::exit(2);
  }
  return rc;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "Usage: %s < input_file >\n", argv[0]);
    return 1;
  }
  const std::vector<Command> cmds = read_input(argv[1]);
  Settings S;
  Topology top;
  sop_engine* eng = nullptr;
  int rep = -1;
  std::vector<double> xyz, unc, vel;
  bool first_run = true;  // the reference's static first_time (sop.cpp:102)
  for (const Command& c : cmds) {
    if (c.cmd == "load") {
      if (!load(c, top)) {
        std::fprintf(stderr, "load %s failed\n", c.opt.empty() ? "" : c.opt[0].c_str());
        return 1;
      }
    } else if (c.cmd == "set") {
      if (c.opt.size() >= 2) S.set(c.opt[0], c.opt[1]);
    } else if (c.cmd == "run") {
      const int n = top.nbead;
      if (n <= 0) {
        std::fprintf(stderr, "run: no initial coordinates loaded\n");
        return 1;
      }
      sop_params p;
      sop_params_default(&p);
      p.T = S.T; p.zeta = S.zeta; p.h = S.h;
      p.a1 = S.a1; p.a2 = S.a2; p.a3 = S.a3; p.a4 = S.a4; p.a5 = S.a5;
      p.boxl = S.boxl; p.lcell = S.lcell; p.ncell = S.ncell;
      p.nnlup = S.nnlup; p.nup = S.nup;
      p.list_mode = S.neighborlist ? SOP_LIST_NEIGHBOR : (S.celllist ? SOP_LIST_CELL : SOP_LIST_NONE);
      p.dynamics = S.sim_type == 2 ? SOP_DYN_OVERDAMPED : SOP_DYN_UNDERDAMPED;
      p.seed = (uint64_t)(int64_t)(-100 - S.run);
      if (!eng) {
        if (top.have_vdw) exclusions(top);
        sop_engine_config cfg;
        sop_engine_config_default(&cfg);
        cfg.max_beads = std::max(2 * n, 4096);
        cfg.max_replicas = 4;
        cfg.max_list_entries = (int64_t)n * 512 + 65536;
        check(sop_engine_create(&cfg, &eng), "sop_engine_create");
        sop_system_desc d;
        std::memset(&d, 0, sizeof d);
        d.nbead = n;
        d.xyz = top.xyz.data();
        top.type.resize(n, 1);
        d.bead_type = top.type.data();
        d.nbnd = (int)top.ib.size(); d.ib = top.ib.data(); d.jb = top.jb.data(); d.r0 = top.r0.data();
        d.nang = (int)top.ia.size(); d.ia = top.ia.data(); d.ka = top.ka.data();
        d.nnat = (int)top.in_.size(); d.in_ = top.in_.data(); d.jn = top.jn.data(); d.rn = top.rn.data();
        d.nexcl = (int)top.ie.size(); d.ie = top.ie.data(); d.je = top.je.data();
        d.params = p;
        check(sop_replica_add(eng, &d, &rep), "sop_replica_add");
        xyz.assign(3 * (size_t)n, 0.0);
        unc.assign(3 * (size_t)n, 0.0);
        vel.assign(3 * (size_t)n, 0.0);
      } else {
        check(sop_replica_set_params(eng, rep, &p), "sop_replica_set_params");
      }
      double istep = 1.0;
      if (S.restart) {  // sop.cpp:132-136: coordinates and velocities from files
        for (const std::string* f : {&S.unccfname, &S.vfname}) {
          if (!read_coords(*f, f == &S.vfname ? vel : unc, n)) {
            std::fprintf(stderr, "restart: cannot read %d beads from %s\n", n, f->c_str());
            return 1;
          }
        }
        check(sop_replica_set_state(eng, rep, unc.data(), vel.data()), "sop_replica_set_state");
        istep = S.istep_restart + 1.0;
        if (S.rgen_restart) check(sop_replica_set_step(eng, rep, (int64_t)S.istep_restart), "set_step");
      }
      if (first_run && !S.rgen_restart) {  // sop.cpp:149-152: the starting frame
        check(sop_replica_get_state(eng, rep, xyz.data(), unc.data(), vel.data()), "get_state");
        append_frame(S.binfname, xyz, n);
        append_frame(S.uncbinfname, unc, n);
      }
      first_run = false;
      const long long nsteps = (long long)(S.nstep - istep + 1.0);
      if (nsteps <= 0) continue;
      FILE* uf = std::fopen(S.ufname.c_str(), "a");
      if (!uf) {
        std::fprintf(stderr, "cannot open %s\n", S.ufname.c_str());
        return 1;
      }
      int status = 0;
      int64_t t0 = 0;  // the replica's step counter: launch L of the window is step t0 + L
      check(sop_replica_status(eng, rep, &status, &t0), "sop_replica_status");
      check(sop_replica_start(eng, rep, nsteps), "sop_replica_start");
      // the window is nsteps + 1 launches (the first evaluates the initial
      // force); the engine computes the output-step energies at steps
      // t % nup == 0, so chunks end right after those launches
      long long done = 0;  // launches completed
      std::vector<int> fin(4);
      int nfin = 0;
      const long long total = nsteps + 1;
      while (done < total) {
        long long next = total;
        if (S.nup > 0) {
          long long L = done;  // first output launch at or after `done`, L >= 1
          if (L < 1) L = 1;
          const long long m = (t0 + L) % S.nup;
          if (m) L += S.nup - m;
          next = std::min(total, L + 1);
        }
        check(sop_run_chunk(eng, next - done, fin.data(), (int)fin.size(), &nfin), "sop_run_chunk");
        done = next;
        const long long L = done - 1;  // the last launch of the chunk
        const long long t = t0 + L;
        if (S.nup > 0 && L > 0 && t % S.nup == 0) {
          double e[6], o[5];
          check(sop_replica_outputs(eng, rep, e, nullptr), "sop_replica_outputs");
          check(sop_observables(eng, rep, o), "sop_observables");
          check(sop_replica_get_state(eng, rep, xyz.data(), unc.data(), vel.data()), "get_state");
          std::fprintf(uf, "%.0lf %f %f %f %f %f %f %f %d %f\n", istep - 1.0 + (double)L, S.T, o[3],
                       e[0], e[1], e[2], e[5], o[0], (int)o[1], o[2]);
          std::fflush(uf);
          append_frame(S.binfname, xyz, n);
          append_frame(S.uncbinfname, unc, n);
          write_coords(S.cfname, xyz, n);
          write_coords(S.unccfname, unc, n);
          write_coords(S.vfname, vel, n);
        }
      }
      std::fclose(uf);
      int64_t steps = 0;
      check(sop_replica_status(eng, rep, &status, &steps), "sop_replica_status");
      if (status) std::fprintf(stderr, "replica status 0x%x after %lld steps\n", status, (long long)steps);
    }
  }
  if (eng) sop_engine_destroy(eng);
  return 0;
}
