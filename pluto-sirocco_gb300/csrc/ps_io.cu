// ps_io.cu -- PLUTO's double-precision snapshot format for device state
// (host code): WriteData's DBL output in single-file mode
// (Src/write_data.c:132-220 with FileWriteData, Src/bin_io.c:216-258) and
// the dbl.out log line (write_data.c:420-448), and reading such a file back
// into a context, as RestartFromFile does for .dbl data (Src/restart.c:104-
// 170).  The layout: every variable in Data.Vc order, each over the active
// cells with x fastest, as native little-endian doubles.  The entropy of
// ENTROPY_SWITCH contexts is not written (Src/set_output.c:177-179); on
// reading it is set from the pressure and density, as the next Boundary()
// would.
#include "ps_ctx.cuh"
#include "ps_physics.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

extern "C" void ps_set_error_msg(const char *msg);

static int io_fail(const std::string &msg)
{
  ps_set_error_msg(msg.c_str());
  return PS_EINVAL;
}

static bool little_endian()
{
  const unsigned one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

static size_t total_cells(const ps_ctx *c)
{
  return (size_t)c->p.ntot[0] * c->p.ntot[1] * c->p.ntot[2];
}

// variables written to / read from .dbl files
static int dumped_vars(const ps_ctx *c) { return c->p.entropy ? c->p.nvar - 1 : c->p.nvar; }

extern "C" int ps_write_dbl(ps_ctx *c, const char *dir, int nfile, const char *names)
{
  if (!c || !dir || nfile < 0) return io_fail("ps_write_dbl: bad arguments");
  if (!little_endian()) return io_fail("ps_write_dbl: big-endian host not supported");
  const ps::Params &p = c->p;
  std::vector<double> V((size_t)p.nvar * total_cells(c));
  int r = ps_get_state(c, V.data());
  if (r < 0) return r;
  char fname[4096];
  std::snprintf(fname, sizeof(fname), "%s/data.%04d.dbl", dir, nfile);
  FILE *f = std::fopen(fname, "wb");
  if (!f) return io_fail(std::string("ps_write_dbl: cannot open ") + fname);
  const size_t plane = (size_t)p.ntot[0] * p.ntot[1];
  bool ok = true;
  for (int nv = 0; nv < dumped_vars(c) && ok; nv++)
    for (int k = p.beg[2]; k < p.beg[2] + p.nx[2] && ok; k++)
      for (int j = p.beg[1]; j < p.beg[1] + p.nx[1] && ok; j++) {
        const double *row = V.data() + nv * total_cells(c) + k * plane + (size_t)j * p.ntot[0] +
                            p.beg[0];
        ok = std::fwrite(row, sizeof(double), (size_t)p.nx[0], f) == (size_t)p.nx[0];
      }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return io_fail(std::string("ps_write_dbl: write failed: ") + fname);

  // dbl.out: the first nfile lines are kept, this snapshot's line follows
  double t = 0.0, dt = 0.0, inv = 0.0;
  long step = 0;
  r = ps_get_time(c, &t, &dt, &step, &inv);
  if (r < 0) return r;
  std::string log;
  char lname[4096];
  std::snprintf(lname, sizeof(lname), "%s/dbl.out", dir);
  if (nfile > 0) {
    FILE *g = std::fopen(lname, "r");  // a missing dbl.out counts as empty
    if (g) {
      char line[1024];
      for (int n = 0; n < nfile && std::fgets(line, sizeof(line), g); n++) log += line;
      std::fclose(g);
    }
  }
  std::string vars;
  if (names && *names) {
    vars = names;
    if (vars.back() != ' ') vars += ' ';
  } else {
    static const char *base[5] = {"rho", "vx1", "vx2", "vx3", "prs"};
    for (int nv = 0; nv < dumped_vars(c); nv++) {
      if (nv < 5)
        vars += base[nv];
      else
        vars += "tr" + std::to_string(nv - 4);
      vars += ' ';
    }
  }
  char head[256];
  std::snprintf(head, sizeof(head), "%d %12.6e %12.6e %ld single_file little ", nfile, t, dt,
                step);
  log += head + vars + "\n";
  FILE *g = std::fopen(lname, "w");
  if (!g) return io_fail(std::string("ps_write_dbl: cannot write ") + lname);
  ok = std::fwrite(log.data(), 1, log.size(), g) == log.size();
  ok = (std::fclose(g) == 0) && ok;
  if (!ok) return io_fail(std::string("ps_write_dbl: write failed: ") + lname);
  return 0;
}

extern "C" int ps_read_dbl(ps_ctx *c, const char *path)
{
  if (!c || !path) return io_fail("ps_read_dbl: bad arguments");
  if (!little_endian()) return io_fail("ps_read_dbl: big-endian host not supported");
  const ps::Params &p = c->p;
  const size_t nact = (size_t)p.nx[0] * p.nx[1] * p.nx[2];
  FILE *f = std::fopen(path, "rb");
  if (!f) return io_fail(std::string("ps_read_dbl: cannot open ") + path);
  std::fseek(f, 0, SEEK_END);
  const long size = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (size != (long)(nact * dumped_vars(c) * sizeof(double))) {
    std::fclose(f);
    return io_fail(std::string("ps_read_dbl: ") + path + " does not hold " +
                   std::to_string(dumped_vars(c)) + " variables over " + std::to_string(nact) +
                   " active cells");
  }
  std::vector<double> V((size_t)p.nvar * total_cells(c));
  int r = ps_get_state(c, V.data());  // keeps the ghost cells; the device refills them
  if (r < 0) {
    std::fclose(f);
    return r;
  }
  const size_t plane = (size_t)p.ntot[0] * p.ntot[1];
  bool ok = true;
  for (int nv = 0; nv < dumped_vars(c) && ok; nv++)
    for (int k = p.beg[2]; k < p.beg[2] + p.nx[2] && ok; k++)
      for (int j = p.beg[1]; j < p.beg[1] + p.nx[1] && ok; j++) {
        double *row = V.data() + nv * total_cells(c) + k * plane + (size_t)j * p.ntot[0] + p.beg[0];
        ok = std::fread(row, sizeof(double), (size_t)p.nx[0], f) == (size_t)p.nx[0];
      }
  std::fclose(f);
  if (!ok) return io_fail(std::string("ps_read_dbl: short read: ") + path);
  if (p.entropy) {
    const size_t n = total_cells(c);
    for (size_t q = 0; q < n; q++)
      V[(p.nvar - 1) * n + q] = V[ps::PRS * n + q] / std::pow(V[ps::RHO * n + q], p.gamma);
  }
  return ps_set_state(c, V.data());
}
