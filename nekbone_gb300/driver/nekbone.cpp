// nekbone -- the reference's driver program (driver.f) over the library's
// Fortran-convention C ABI, for hosts without a Fortran compiler.
//
// It reads the case's data.rea (read_param, driver.f:402-484) and, for every
// polynomial order and element count of the requested ranges, makes the
// driver's calls in the driver's order (driver.f:38-67): init_mesh,
// proxy_setupds, set_multiplicity, proxy_setup, h1mg_setup, set_f, the
// warm-up cg, then the timed cg bracketed by set_timer_flop_cnt, and gs_free.
// Output lines follow the reference's formats (cg.f:44,79 and
// driver.f:307-318).  One process, one GPU: np = 1.
//
// Usage: nekbone [data.rea] [--mgrid] [--digits]
//   --mgrid   the hsmg preconditioner (the reference's MGRID build)
//   --digits  print the cg norms with 17 significant digits
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/nekbone_gb300.h"

namespace {

bool g_digits = false;

double wall() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// data.rea: five records (driver.f:415-420); anything after the values on
// a line is a comment.
bool read_param(const char *path, bool *ifbrick, int v[12]) {
  std::ifstream in(path);
  if (!in) return false;
  std::string line;
  std::vector<std::string> rec;
  while (std::getline(in, line) && rec.size() < 5) rec.push_back(line);
  if (rec.size() < 5) return false;
  {
    std::istringstream s(rec[0]);
    std::string b;
    s >> b;
    for (auto &ch : b) ch = char(std::tolower(ch));
    if (b.find("t") != std::string::npos) *ifbrick = true;
    else if (b.find("f") != std::string::npos) *ifbrick = false;
    else return false;
  }
  for (int r = 1; r < 5; ++r) {
    std::istringstream s(rec[r]);
    for (int k = 0; k < 3; ++k)
      if (!(s >> v[3 * (r - 1) + k])) return false;
  }
  return true;
}

bool check(const char *what) {
  const int st = nekbone_last_status();
  if (st) {
    std::fprintf(stderr, "%s failed: %s\n", what, nekbone_last_message());
    return false;
  }
  return true;
}

// cubic (driver.f:196-247) through the library's restatement
void cubic(int *mx, int *my, int *mz, int np) { cubic_(mx, my, mz, &np); }

void print_cg(int iter, int nvals, const double *vals) {
  std::printf("cg:%4d", iter);
  for (int k = 0; k < nvals; ++k) {
    if (g_digits) std::printf(" %.17E", vals[k]);
    else std::printf("%12.4E", vals[k]);
  }
  std::printf("\n");
}

}  // namespace

int main(int argc, char **argv) {
  const char *rea = "data.rea";
  bool mgrid = false;
  for (int a = 1; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--mgrid")) mgrid = true;
    else if (!std::strcmp(argv[a], "--digits")) g_digits = true;
    else rea = argv[a];
  }
  nekbone_set_error_mode(1);
  bool ifbrick = false;
  int v[12];
  if (!read_param(rea, &ifbrick, v)) {
    std::printf(" ERROR READING    data.rea.....ABORT\n");
    std::printf(" CHECK PARAMETERS data.rea.....ABORT\n");
    return 0;
  }
  int iel0 = v[0], ielN = v[1], ielD = v[2], nx0 = v[3], nxN = v[4], nxD = v[5];
  int npx = v[6], npy = v[7], npz = v[8], mx = v[9], my = v[10], mz = v[11];
  if (iel0 > ielN || nx0 > nxN) {
    std::printf(" ERROR data.rea :: iel0 > ielN or nx0 > nxN :: ABORT\n");
    return 0;
  }
  if (ielD > ielN || nxD > nxN) std::printf(" WARNING data.rea : STRIDE   nxD>nxN or ielD>ielN !!!\n");
  if (nx0 < 4 && mgrid) {
    std::printf(" ERROR data.rea nx0 must be greater than or equal to 4 ...setting nx0=4\n");
    nx0 = 4;
  }
  if (ielD < 1) ielD = 1;
  if (nxD < 1) nxD = 1;
  std::printf(" ifmgrid    : %c    ifbrick    : %c\n", mgrid ? 'T' : 'F', ifbrick ? 'T' : 'F');
  const int mask_mode = 0, mg = mgrid ? 1 : 0;
  nekbone_set_mask_mode_(&mask_mode);       // the reference's maskit
  nekbone_set_mgrid_(&mg);

  const int np = 1;
  std::vector<double> mflops_list;
  for (int nx1 = nx0; nx1 <= nxN; nx1 += nxD) {
    for (int nelt = iel0; nelt <= ielN; nelt += ielD) {
      // init_mesh (driver.f:117-194)
      int nelx, nely, nelz;
      if (!ifbrick) {
        nelx = nelt * np, nely = 1, nelz = 1;
        npx = np, npy = 1, npz = 1;
        mx = nelt, my = 1, mz = 1;
      } else {
        if (npx * npy * npz != np) cubic(&npx, &npy, &npz, np);
        if (mx * my * mz != nelt) cubic(&mx, &my, &mz, nelt);
        nelx = mx * npx, nely = my * npy, nelz = mz * npz;
      }
      std::printf("\n Processor Distribution:  npx,npy,npz= %11d %11d %11d\n", npx, npy, npz);
      std::printf(" Element Distribution: nelx,nely,nelz= %11d %11d %11d\n", nelx, nely, nelz);
      std::printf(" Local Element Distribution: mx,my,mz= %11d %11d %11d\n", mx, my, mz);
      std::vector<int> lglel(nelt);
      {
        int e = 0;
        for (int k = 0; k < mz; ++k)
          for (int j = 0; j < my; ++j)
            for (int i = 0; i < mx; ++i) lglel[e++] = i + j * nelx + k * nelx * nely + 1;
      }
      const int n = nelt * nx1 * nx1 * nx1;
      // proxy_setup's semhat first: /dxyz/ dxm1 is published with the mesh
      std::vector<double> ah(nx1 * nx1), bh(nx1), ch(nx1 * nx1), dh(nx1 * nx1), zh(nx1),
          wh(2 * nx1);
      const int nn = nx1 - 1;
      semhat_(ah.data(), bh.data(), ch.data(), dh.data(), zh.data(), wh.data(), &nn);
      int gsh = -1;
      nekbone_common_(&nelx, &nely, &nelz, &nelt, &nx1, lglel.data(), dh.data(), &gsh);
      nekbone_mask_reset_();
      if (!check("init_mesh")) return 1;
      // proxy_setupds (prox_dssum.f:14-40)
      std::vector<int64_t> glo(n);
      set_vert_box_(glo.data(), &nx1);
      const int zero = 0, one = 1;
      gs_setup_(&gsh, glo.data(), &n, &zero, &one);
      if (!check("proxy_setupds")) return 1;
      nekbone_common_(&nelx, &nely, &nelz, &nelt, &nx1, lglel.data(), dh.data(), &gsh);
      std::vector<double> c(n), g(6 * size_t(n)), f(n), x(n), r(n), w(n), p(n), z(n);
      set_multiplicity_(c.data());
      setup_g_(g.data());
      h1mg_setup_();
      set_f_(f.data(), c.data(), &n);
      if (!check("set-up")) return 1;
      const int niter = 100;
      double flop_cg = 0.0;
      auto run_cg = [&]() -> bool {
        cg_(x.data(), f.data(), g.data(), c.data(), r.data(), w.data(), p.data(), z.data(), &n,
            &niter, &flop_cg);
        if (!check("cg")) return false;
        int it = 0;
        double r0 = 0, rn = 0, al = 0, be = 0, pa = 0;
        nekbone_cg_report_(&it, &r0, &rn, &al, &be, &pa);
        const double first[1] = {r0};
        print_cg(0, 1, first);
        const double last[4] = {rn, al, be, pa};
        print_cg(it, 4, last);
        return true;
      };
      std::printf("\n");
      if (!run_cg()) return 1;
      // set_timer_flop_cnt(0) / (1) (driver.f:293-322)
      const double fz = 0.0;
      nekbone_set_flops_(&fz, &fz);
      flop_cg = 0.0;
      const double t0 = wall();
      if (!run_cg()) return 1;
      const double time1 = wall() - t0;
      double flop_a = 0.0, fcg = 0.0;
      nekbone_get_flops_(&flop_a, &fcg);
      double mflops = 0.0;
      if (time1 > 0) mflops = (flop_a + flop_cg) / (1.e6 * time1);
      std::printf("\n");
      std::printf("nelt = %7d, np = %9d, nx1 = %7d, elements =%10d\n", nelt, np, nx1, nelt * np);
      std::printf("Tot MFlops = %12.4E, MFlops      = %12.4E\n", mflops * np, mflops);
      std::printf("Setup Flop = %12.4E, Solver Flop = %12.4E\n", flop_a, flop_cg);
      std::printf("Solve Time = %12.4E\n", time1);
      gs_free_(&gsh);
      if (!check("gs_free")) return 1;
      mflops_list.push_back(mflops * np);
    }
  }
  double avg = 0.0;
  for (double m : mflops_list) avg += m;
  if (!mflops_list.empty()) avg /= double(mflops_list.size());
  std::printf("Avg MFlops = %12.4E\n", avg);
  return 0;
}
