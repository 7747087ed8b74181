// ORACLE -- test infrastructure only, never part of the product path.
//
// A serial CPU restatement of the ADPRES static k-eigenvalue path, written to
// follow the reference's loops, evaluation order and single-precision default
// literals so that its output can be compared with the reference's own printed
// IAEA3D convergence trace (docs/quick-guides.md:161-191) digit for digit.
// It is used only by tests/, __graft_entry__.smoke() and the CPU-baseline leg
// of bench.py, as the checker of the CUDA path.
//
// Every routine cites the reference routine it restates (path:line inside the
// ADPRES project).  Build with -ffp-contract=off: the reference is compiled by
// gfortran for x86-64 without FMA, so no multiply-add may be fused here.
//
// Scope: deck cards %MODE %CASE %XSEC %GEOM %ADF %ITER %KERN %PRNT (+ FILE
// includes, '!' comments), the feedback cards %CROD %CBCS %BCON %FTEM %MTEM
// %CDEN and the transient cards %EJCT %THET %EXTR; XS_updt (base, state and
// rod updates, D/sigr, checks); forward `outer` and adjoint `outer_ad` with
// BiCGSTAB, fission-source extrapolation and the SANM/PNM two-node nodal
// update; PowDis and the AsmPow/AxiPow/AsmFlux edits; reactivity and
// calc_beta; the critical boron search cbsearch; the rod ejection transient
// (rod_eject, trans_calc, outer_tr, KNE1).  Reference STOPs become error
// codes.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include <algorithm>
#include <cctype>
#include <chrono>

namespace {

// Status codes shared in meaning with the product's adp_status.
enum {
  ORA_OK = 0,
  ORA_ERR_INPUT = 1,
  ORA_ERR_BADXS = 2,
  ORA_ERR_PIVOT = 3,
  ORA_ERR_DIVERGED = 4,
  ORA_ERR_MAXOUTER = 5,
  ORA_ERR_ZEROPOWER = 6,
  ORA_ERR_UNSUPPORTED = 7,
};

struct OraError : std::runtime_error {
  int code;
  OraError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Single-precision default literals of the reference, promoted to double the
// way gfortran promotes them in mixed-kind expressions.
const double F_1em5 = (double)1.e-5f;   // mod_data.f90:78-79, mod_xsec.f90:216
const double F_1em2 = (double)1.e-2f;   // mod_cmfd.f90:495
const double F_1em4 = (double)10e-5f;   // mod_nodal.f90:856
const double F_1em20 = (double)1.e-20f; // mod_xsec.f90:112

struct TraceRec {
  int p;
  double k, ser, fer;
  int extrapolated;
  int nodal;           // 1 if a nodal update happened in this outer
  double ndmax;
  int im, jm, km;
};

struct Ora {
  std::string err;
  // ---- cards -------------------------------------------------------------
  std::string mode;
  std::string kern = "SANM";            // right-adjusted 4 characters
  int ng = 0, nmat = 0;
  std::vector<double> xsigtr, xsiga, xnuf, xsigf, chi, xsigs;   // (nmat,ng[,ng])
  int nx = 0, ny = 0, nz = 0, nxx = 0, nyy = 0, nzz = 0, nnod = 0;
  std::vector<double> xsize, ysize, zsize, xdel, ydel, zdel, vdel;
  std::vector<int> xdiv, ydiv, zdiv;
  int np = 0;
  std::vector<int> zpln;
  std::vector<std::vector<int>> pasm;   // per planar: (nx,ny)
  std::vector<int> mnum;                // (nxx,nyy,nzz)
  std::vector<int> ysmin, ysmax, xsmin, xsmax;  // ystag(nyy), xstag(nxx)
  int xeast = 0, xwest = 0, ynorth = 0, ysouth = 0, zbott = 0, ztop = 0;
  std::vector<int> ix, iy, iz, xyz, mat;
  // iteration control (mod_data.f90:78-86)
  double ferc = F_1em5, serc = F_1em5;
  int nin = 2, nout = 500, nac = 5, th_niter = 30, nth = 20, nupd = 0;
  int aprad = 1, apaxi = 1, afrad = 1;
  bool badf = false;
  // cross-section feedback cards (mod_io.f90:2148-2954): per-material changes
  // (nmat,ng[,ng]) per unit of a state variable
  struct Feedback {
    bool on = false;
    double ref = 0.0, val = 0.0;                        // reference and current value
    std::vector<double> str, sa, nf, sf, ss;            // sigtr siga nuf sigf sigs changes
  };
  Feedback fb_bcon, fb_ftem, fb_mtem, fb_cden, fb_crod;  // fb_crod.ss etc.: per fully rodded node
  bool bcbcs = false;                                   // %CBCS (critical boron search) rather than %BCON
  int nb = 0, nstep = 0;
  double pos0 = 0.0, ssize = 0.0, coreh = 0.0;
  std::vector<double> bpos;                             // (nb) bank positions in steps
  std::vector<int> fbmap;                               // (nxx,nyy) bank of each node column, 0 none
  double bcon = 0.0;                                    // %BCON concentration (forward mode)
  // rod ejection transient (%EJCT, %THET, %EXTR; mod_io.f90:1650-1689,
  // 2332-2482): bank motion, time steps, delayed neutron data, velocities
  static constexpr int nf = 6;                          // precursor families (mod_data.f90:131)
  double ibeta[nf] = {0, 0, 0, 0, 0, 0}, lamb[nf] = {0, 0, 0, 0, 0, 0};
  std::vector<double> velo;                             // (ng)
  double ttot = 0.0, tstep1 = 0.0, tdiv = 0.0, tstep2 = 0.0;
  std::vector<double> fbpos, tmove, bspeed;             // (nb)
  std::vector<int> mdir;                                // 0 still, 1 down, 2 up
  double sth = 1.0, bth = 0.0;                          // theta and (1 - theta) / theta
  bool bextr = false;                                   // exponential flux transformation
  // transient state (mod_trans.f90, mod_cmfd.f90:800-952)
  std::vector<double> c0;                               // (nnod,nf) precursor densities
  std::vector<double> omeg, Lt, ft, sigrp;              // (nnod,ng) frequencies, leakage, old flux, removal
  std::vector<double> fst, dfis;                        // (nnod)
  std::vector<double> tbeta;                            // (nmat)
  double ctbeta = 0.0;
  std::vector<double> dc;               // (nnod,ng,6)
  std::vector<double> exsrc;            // (nnod,ng)
  // node XS
  std::vector<double> sigtr, siga, nuf, sigf, sigs, D, sigr;
  // solver state
  std::vector<double> df, dn;           // (nnod,ng,6)  NODE_DATA
  std::vector<double> Amat;             // (7,nnod,ng): elmn(1..ncol)
  std::vector<int> ncol, col;           // ind(n)%ncol, ind(n)%col(7)
  std::vector<double> f0, fs0, s0;
  double Ke = 0.0, ndmax = 0.0;
  int im = 0, jm = 0, km = 0;
  bool coup_first = true, matrix_first = true, outer_first = true, outer_ad_first = true;
  bool source_first = true;
  // nodal module state (mod_nodal.f90:7-12, mod_data.f90:196-201)
  int cmode = 1;
  std::vector<double> Bcn, Bcp, An, Bn, En, Fn, Gn, Hn, Ap, Bp, Ep, Fp, Gp, Hp, Lm2;
  std::vector<double> S1, S2, S3;
  std::vector<double> a1n, a2n, a3n, a4n, a1p, a2p, a3p, a4p, Ln1, Lp1;
  // trace of the last outer call
  std::vector<TraceRec> trace;
  int last_outers = 0;
  double last_ser = 0, last_fer = 0;
  double t_cmfd = 0, t_nodal = 0;

  // 1-based Fortran-layout accessors
  inline double& X3(std::vector<double>& a, int n, int g, int u) { return a[(n - 1) + (size_t)nnod * ((g - 1) + (size_t)ng * (u - 1))]; }
  inline double& N2(std::vector<double>& a, int n, int g) { return a[(n - 1) + (size_t)nnod * (g - 1)]; }
  inline double& M2(std::vector<double>& a, int i, int g) { return a[(i - 1) + (size_t)nmat * (g - 1)]; }
  inline double& M3(std::vector<double>& a, int i, int g, int h) { return a[(i - 1) + (size_t)nmat * ((g - 1) + (size_t)ng * (h - 1))]; }
  inline double& SG(std::vector<double>& a, int n, int g, int h) { return a[(n - 1) + (size_t)nnod * ((g - 1) + (size_t)ng * (h - 1))]; }
  inline int& XYZ(int i, int j, int k) { return xyz[(i - 1) + (size_t)nxx * ((j - 1) + (size_t)nyy * (k - 1))]; }
  inline int& MN(int i, int j, int k) { return mnum[(i - 1) + (size_t)nxx * ((j - 1) + (size_t)nyy * (k - 1))]; }
  inline double& Bm(std::vector<double>& a, int g, int h) { return a[(g - 1) + (size_t)ng * (h - 1)]; }
  inline double& AE(int i, int n, int g) { return Amat[(i - 1) + 7 * ((n - 1) + (size_t)nnod * (g - 1))]; }
  inline int& COL(int n, int i) { return col[(i - 1) + 7 * (size_t)(n - 1)]; }
};

// ===========================================================================
// Deck reading (mod_io.f90)
// ===========================================================================

struct Line { int ln; std::string text; };

static std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

static std::string upper(std::string s) {
  for (auto& c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

// inp_comments (mod_io.f90:452-492): drop blank lines, whole-line comments and
// the tail after '!'.
static void strip_comments(const std::string& text, std::vector<Line>& out) {
  std::istringstream is(text);
  std::string raw;
  int ln = 0;
  while (std::getline(is, raw)) {
    ++ln;
    if (raw.size() > 200) raw = raw.substr(0, 200);
    for (auto& c : raw) if (c == '\t') c = ' ';
    std::string l = trim(raw);
    size_t comm = l.find('!');
    if (comm == std::string::npos) {
      if (!l.empty()) out.push_back({ln, l});
    } else if (comm > 0) {
      out.push_back({ln, l.substr(0, comm)});
    }
  }
}

static std::string read_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw OraError(ORA_ERR_INPUT, "cannot open file: " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

static std::string dirname_of(const std::string& p) {
  size_t s = p.find_last_of('/');
  return s == std::string::npos ? std::string(".") : p.substr(0, s);
}

// inp_rewrite (mod_io.f90:496-576): split the buffer into cards, honouring
// the FILE include keyword.
struct Cards {
  std::vector<std::pair<std::string, std::vector<Line>>> cards;
  std::vector<Line>* find(const std::string& name) {
    for (auto& c : cards) if (c.first == name) return &c.second;
    return nullptr;
  }
};

static void split_cards(const std::vector<Line>& buf, const std::string& basedir, Cards& cards) {
  static const char* known[] = {"MODE", "XSEC", "GEOM", "CASE", "ESRC", "ITER", "PRNT", "ADF",
                                "CROD", "EJCT", "CBCS", "FTEM", "MTEM", "CDEN", "BCON", "THER",
                                "XTAB", "KERN", "EXTR", "THET"};
  std::vector<Line>* cur = nullptr;
  for (const auto& L : buf) {
    if (L.text.find("FILE") != std::string::npos || L.text.find("file") != std::string::npos) {
      std::string l = trim(L.text);
      size_t sp = l.find(' ');
      std::string fname = sp == std::string::npos ? std::string("") : trim(l.substr(sp + 1));
      std::string content;
      std::ifstream t1(fname);
      std::ifstream t2(basedir + "/" + fname);
      if (t1) content = read_file(fname);
      else if (t2 || fname.empty() || fname[0] != '/') content = read_file(basedir + "/" + fname);
      else content = read_file(basedir + "/" + fname.substr(fname.rfind('/') + 1));   // another machine's absolute path
      std::vector<Line> inc;
      strip_comments(content, inc);
      if (!cur) throw OraError(ORA_ERR_INPUT, "FILE include outside a card");
      for (auto& x : inc) cur->push_back(x);
    }
    size_t per = L.text.find('%');
    if (per != std::string::npos) {
      std::string name = trim(L.text.substr(per + 1));
      bool ok = false;
      for (auto k : known) if (name == k) ok = true;
      if (!ok) throw OraError(ORA_ERR_INPUT, "line " + std::to_string(L.ln) + ": wrong input card: " + name);
      cards.cards.push_back({name, {}});
      cur = &cards.cards.back().second;
      continue;
    }
    if (!cur) continue;   // text before the first card is ignored
    if (L.text.find("FILE") != std::string::npos || L.text.find("file") != std::string::npos) continue;
    cur->push_back(L);
  }
}

// Fortran list-directed input of one record: blanks/commas separate values,
// r*v repeats, '/' ends the record.
struct Rec {
  std::vector<std::string> toks;
  size_t pos = 0;
  int ln = 0;
  std::string card;
  explicit Rec(const Line& L, const std::string& c) : ln(L.ln), card(c) {
    std::string s = L.text;
    size_t slash = s.find('/');
    if (slash != std::string::npos) s = s.substr(0, slash);
    for (auto& ch : s) if (ch == ',') ch = ' ';
    std::istringstream is(s);
    std::string t;
    while (is >> t) {
      size_t st = t.find('*');
      if (st != std::string::npos && st > 0) {
        int r = std::atoi(t.substr(0, st).c_str());
        std::string v = t.substr(st + 1);
        for (int q = 0; q < r; ++q) toks.push_back(v);
      } else {
        toks.push_back(t);
      }
    }
  }
  [[noreturn]] void fail(const std::string& what) {
    throw OraError(ORA_ERR_INPUT, "card %" + card + " line " + std::to_string(ln) + ": " + what);
  }
  const std::string& next() {
    if (pos >= toks.size()) fail("this line needs more input data");
    return toks[pos++];
  }
  int geti() {
    const std::string& t = next();
    char* e = nullptr;
    long v = std::strtol(t.c_str(), &e, 10);
    if (e == t.c_str() || *e != '\0') fail("bad integer '" + t + "'");
    return (int)v;
  }
  double getd() {
    std::string t = next();
    for (auto& c : t) if (c == 'd' || c == 'D') c = 'e';
    char* e = nullptr;
    double v = std::strtod(t.c_str(), &e);
    if (e == t.c_str() || *e != '\0') fail("bad real '" + t + "'");
    return v;
  }
};

struct CardReader {
  std::vector<Line>* lines;
  size_t i = 0;
  std::string name;
  CardReader(std::vector<Line>* l, const std::string& n) : lines(l), name(n) {}
  bool more() const { return i < lines->size(); }
  Rec rec() {
    if (i >= lines->size()) throw OraError(ORA_ERR_INPUT, "card %" + name + ": unexpected end of card");
    return Rec((*lines)[i++], name);
  }
};

// inp_xsec (mod_io.f90:683-805)
static void read_xsec(Ora& o, std::vector<Line>* L) {
  CardReader cr(L, "XSEC");
  Rec r = cr.rec();
  o.ng = r.geti();
  o.nmat = r.geti();
  if (o.ng < 1 || o.nmat < 1) r.fail("bad group or material count");
  o.xsigtr.assign((size_t)o.nmat * o.ng, 0);
  o.xsiga = o.xnuf = o.xsigf = o.chi = o.xsigtr;
  o.xsigs.assign((size_t)o.nmat * o.ng * o.ng, 0);
  for (auto& l : *L) if (l.text.find('/') != std::string::npos || l.text.find('\\') != std::string::npos)
    throw OraError(ORA_ERR_INPUT, "slash or backslash not accepted in %XSEC card");
  bool ccnuf = true, ccsigf = true;
  for (int i = 1; i <= o.nmat; ++i) {
    for (int g = 1; g <= o.ng; ++g) {
      Rec x = cr.rec();
      o.M2(o.xsigtr, i, g) = x.getd();
      o.M2(o.xsiga, i, g) = x.getd();
      o.M2(o.xnuf, i, g) = x.getd();
      o.M2(o.xsigf, i, g) = x.getd();
      o.M2(o.chi, i, g) = x.getd();
      for (int h = 1; h <= o.ng; ++h) o.M3(o.xsigs, i, g, h) = x.getd();
      if (o.M2(o.xsigtr, i, g) <= 0.0)
        throw OraError(ORA_ERR_BADXS, "transport cross section is zero or negative in material " +
                                          std::to_string(i) + " group " + std::to_string(g));
      if (o.M2(o.xnuf, i, g) > 0.) ccnuf = false;
      if (o.M2(o.xsigf, i, g) > 0.) ccsigf = false;
    }
  }
  if (ccnuf) throw OraError(ORA_ERR_BADXS, "the problem has no fission material (nu*fission all zero)");
  if (ccsigf) throw OraError(ORA_ERR_BADXS, "the problem has no fission material (fission xsec all zero)");
}

// inp_geom1 (mod_io.f90:809-954)
static void read_geom(Ora& o, std::vector<Line>* L) {
  CardReader cr(L, "GEOM");
  Rec r = cr.rec();
  o.nx = r.geti(); o.ny = r.geti(); o.nz = r.geti();
  if (o.nx < 2) r.fail("nx shall be at least 2");
  if (o.ny < 2) r.fail("ny shall be at least 2");
  if (o.nz < 2) r.fail("nz shall be at least 2");
  if (o.nx > 33) r.fail("nx shall be maximum 33");
  if (o.ny > 33) r.fail("ny shall be maximum 33");
  if (o.nz > 40) r.fail("nz shall be maximum 40");
  auto rdv = [&](std::vector<double>& v, int n) { Rec q = cr.rec(); v.resize(n); for (int i = 0; i < n; ++i) v[i] = q.getd(); };
  auto rdi = [&](std::vector<int>& v, int n) { Rec q = cr.rec(); v.resize(n); for (int i = 0; i < n; ++i) v[i] = q.geti(); };
  rdv(o.xsize, o.nx); rdi(o.xdiv, o.nx);
  rdv(o.ysize, o.ny); rdi(o.ydiv, o.ny);
  rdv(o.zsize, o.nz); rdi(o.zdiv, o.nz);
  o.nxx = o.nyy = o.nzz = 0;
  for (int i = 0; i < o.nx; ++i) { if (o.xdiv[i] < 1) r.fail("division must be >= 1"); o.nxx += o.xdiv[i]; }
  for (int j = 0; j < o.ny; ++j) { if (o.ydiv[j] < 1) r.fail("division must be >= 1"); o.nyy += o.ydiv[j]; }
  for (int k = 0; k < o.nz; ++k) { if (o.zdiv[k] < 1) r.fail("division must be >= 1"); o.nzz += o.zdiv[k]; }
  if (o.nxx > 800) r.fail("nxx shall be maximum 800");
  if (o.nyy > 800) r.fail("nyy shall be maximum 800");
  if (o.nzz > 800) r.fail("nzz shall be maximum 800");
  auto deltas = [](const std::vector<double>& size, const std::vector<int>& div, std::vector<double>& del) {
    del.clear();
    for (size_t i = 0; i < size.size(); ++i) {
      double d = size[i] / (double)(float)div[i];
      for (int l = 0; l < div[i]; ++l) del.push_back(d);
    }
  };
  deltas(o.xsize, o.xdiv, o.xdel);
  deltas(o.ysize, o.ydiv, o.ydel);
  deltas(o.zsize, o.zdiv, o.zdel);

  // inp_geom2 (mod_io.f90:958-1289)
  Rec q = cr.rec();
  o.np = q.geti();
  rdi(o.zpln, o.nz);
  for (int k = 0; k < o.nz; ++k) {
    if (o.zpln[k] > o.np) r.fail("planar is greater than number of planar");
    if (o.zpln[k] < 1) r.fail("planar should be at least 1");
  }
  o.pasm.assign(o.np, std::vector<int>((size_t)o.nx * o.ny, 0));
  for (int k = 0; k < o.np; ++k)
    for (int j = o.ny; j >= 1; --j) {   // north row first
      Rec m = cr.rec();
      for (int i = 1; i <= o.nx; ++i) o.pasm[k][(i - 1) + (size_t)o.nx * (j - 1)] = m.geti();
    }
  o.mnum.assign((size_t)o.nxx * o.nyy * o.nzz, 0);
  int ztot = 0;
  for (int k = 1; k <= o.nz; ++k)
    for (int lz = 1; lz <= o.zdiv[k - 1]; ++lz) {
      ++ztot;
      int ytot = 0;
      for (int j = 1; j <= o.ny; ++j)
        for (int ly = 1; ly <= o.ydiv[j - 1]; ++ly) {
          ++ytot;
          int xtot = 0;
          for (int i = 1; i <= o.nx; ++i)
            for (int lx = 1; lx <= o.xdiv[i - 1]; ++lx) {
              ++xtot;
              int m = o.pasm[o.zpln[k - 1] - 1][(i - 1) + (size_t)o.nx * (j - 1)];
              if (m > o.nmat) throw OraError(ORA_ERR_INPUT, "material is greater than number of material");
              if (m < 0) throw OraError(ORA_ERR_INPUT, "negative material found");
              o.MN(xtot, ytot, ztot) = m;
            }
        }
    }
  o.ysmin.assign(o.nyy, 0); o.ysmax.assign(o.nyy, 0);
  o.xsmin.assign(o.nxx, 0); o.xsmax.assign(o.nxx, 0);
  for (int j = 1; j <= o.nyy; ++j) {
    o.ysmin[j - 1] = o.nxx;
    for (int i = 1; i <= o.nxx; ++i) if (o.MN(i, j, 1) != 0) { o.ysmin[j - 1] = i; break; }
    o.ysmax[j - 1] = 0;
    for (int i = o.nxx; i >= 1; --i) if (o.MN(i, j, 1) != 0) { o.ysmax[j - 1] = i; break; }
  }
  for (int i = 1; i <= o.nxx; ++i) {
    o.xsmin[i - 1] = o.nyy;
    for (int j = 1; j <= o.nyy; ++j) if (o.MN(i, j, 1) != 0) { o.xsmin[i - 1] = j; break; }
    o.xsmax[i - 1] = 0;
    for (int j = o.nyy; j >= 1; --j) if (o.MN(i, j, 1) != 0) { o.xsmax[i - 1] = j; break; }
  }
  for (int k = 1; k <= o.nzz; ++k)
    for (int j = 1; j <= o.nyy; ++j)
      for (int i = o.ysmin[j - 1]; i <= o.ysmax[j - 1]; ++i)
        if (o.MN(i, j, k) == 0) throw OraError(ORA_ERR_INPUT, "zero material found inside core");
  for (int k = 1; k <= o.nzz; ++k)
    for (int i = 1; i <= o.nxx; ++i)
      for (int j = o.xsmin[i - 1]; j <= o.xsmax[i - 1]; ++j)
        if (o.MN(i, j, k) == 0) throw OraError(ORA_ERR_INPUT, "zero material found inside core");
  // The two-node sweeps (mod_nodal.f90:53-125) and the transverse-leakage
  // moments (mod_nodal.f90:1047-1341) need every x row, y column and z line to
  // hold at least two nodes; the reference reads outside its arrays otherwise.
  for (int j = 1; j <= o.nyy; ++j)
    if (o.ysmax[j - 1] - o.ysmin[j - 1] < 1) throw OraError(ORA_ERR_INPUT, "x row with fewer than two nodes");
  for (int i = 1; i <= o.nxx; ++i)
    if (o.xsmax[i - 1] - o.xsmin[i - 1] < 1) throw OraError(ORA_ERR_INPUT, "y column with fewer than two nodes");
  Rec bc = cr.rec();
  o.xeast = bc.geti(); o.xwest = bc.geti(); o.ynorth = bc.geti();
  o.ysouth = bc.geti(); o.zbott = bc.geti(); o.ztop = bc.geti();
  int bcs[6] = {o.xeast, o.xwest, o.ynorth, o.ysouth, o.zbott, o.ztop};
  for (int b : bcs) if (b > 2 || b < 0) bc.fail("wrong boundary conditions");
  o.nnod = 0;
  for (int k = 1; k <= o.nzz; ++k)
    for (int j = 1; j <= o.nyy; ++j)
      for (int i = o.ysmin[j - 1]; i <= o.ysmax[j - 1]; ++i) ++o.nnod;
}

// misc (mod_io.f90:1293-1365)
static void misc(Ora& o) {
  o.ix.assign(o.nnod, 0); o.iy = o.ix; o.iz = o.ix; o.mat = o.ix;
  o.xyz.assign((size_t)o.nxx * o.nyy * o.nzz, 0);
  int n = 0;
  for (int k = 1; k <= o.nzz; ++k)
    for (int j = 1; j <= o.nyy; ++j)
      for (int i = o.ysmin[j - 1]; i <= o.ysmax[j - 1]; ++i) {
        ++n;
        o.ix[n - 1] = i; o.iy[n - 1] = j; o.iz[n - 1] = k;
        o.XYZ(i, j, k) = n;
        o.mat[n - 1] = o.MN(i, j, k);
      }
  size_t nn = (size_t)o.nnod * o.ng;
  o.sigtr.assign(nn, 0); o.siga = o.nuf = o.sigf = o.D = o.sigr = o.sigtr;
  o.sigs.assign(nn * o.ng, 0);
  o.vdel.assign(o.nnod, 0);
  for (int i = 1; i <= o.nnod; ++i)
    o.vdel[i - 1] = o.xdel[o.ix[i - 1] - 1] * o.ydel[o.iy[i - 1] - 1] * o.zdel[o.iz[i - 1] - 1];
  o.ncol.assign(o.nnod, 0);
  o.col.assign((size_t)o.nnod * 7, 0);
  for (int m = 1; m <= o.nnod; ++m) {
    int noz = 0, i = o.ix[m - 1], j = o.iy[m - 1], k = o.iz[m - 1];
    if (k != 1) ++noz;
    if (j != o.xsmin[i - 1]) ++noz;
    if (i != o.ysmin[j - 1]) ++noz;
    ++noz;
    if (i != o.ysmax[j - 1]) ++noz;
    if (j != o.xsmax[i - 1]) ++noz;
    if (k != o.nzz) ++noz;
    o.ncol[m - 1] = noz;
  }
  // nupd = ceiling((nxx + nyy + nzz) / 2.5): integer / default real
  float q = (float)(o.nxx + o.nyy + o.nzz) / 2.5f;
  o.nupd = (int)std::ceil(q);
}

// inp_iter (mod_io.f90:1522-1569)
static void read_iter(Ora& o, std::vector<Line>* L) {
  CardReader cr(L, "ITER");
  Rec r = cr.rec();
  o.nout = r.geti(); o.nin = r.geti(); o.serc = r.getd(); o.ferc = r.getd();
  o.nac = r.geti(); o.nupd = r.geti(); o.th_niter = r.geti(); o.nth = r.geti();
  if (o.nout < o.nupd && o.kern != " FDM")
    r.fail("max. number of outer iteration should be bigger than nodal update interval");
}

// inp_kern (mod_io.f90:1593-1646)
static void read_kern(Ora& o, std::vector<Line>* L) {
  CardReader cr(L, "KERN");
  Rec r = cr.rec();
  std::string k = r.next();
  if (k.size() > 4) k = k.substr(0, 4);
  while (k.size() < 4) k = " " + k;
  if (k != " FDM" && k != " PNM" && k != "SANM") r.fail("could not recognize nodal kernel: " + k);
  o.kern = k;
}

// inp_adf (mod_io.f90:1732-2104) with rotate (mod_io.f90:2108-2144)
static void read_adf(Ora& o, std::vector<Line>* L) {
  CardReader cr(L, "ADF");
  std::vector<double> mdc((size_t)o.nmat * o.ng * 6);
  for (int i = 1; i <= o.nmat; ++i)
    for (int g = 1; g <= o.ng; ++g) {
      Rec r = cr.rec();
      for (int j = 1; j <= 6; ++j) mdc[(j - 1) + 6 * ((i - 1) + (size_t)o.nmat * (g - 1))] = r.getd();
    }
  auto XDC = [&](std::vector<double>& a, int i, int j, int k, int g, int u) -> double& {
    return a[(u - 1) + 6 * ((i - 1) + (size_t)o.nx * ((j - 1) + (size_t)o.ny * ((k - 1) + (size_t)o.nz * (g - 1))))];
  };
  std::vector<double> xdc((size_t)6 * o.nx * o.ny * o.nz * o.ng, 0.0);
  for (int g = 1; g <= o.ng; ++g)
    for (int k = 1; k <= o.nz; ++k)
      for (int j = 1; j <= o.ny; ++j)
        for (int i = 1; i <= o.nx; ++i) {
          int m = o.pasm[o.zpln[k - 1] - 1][(i - 1) + (size_t)o.nx * (j - 1)];
          if (m != 0)
            for (int u = 1; u <= 6; ++u) XDC(xdc, i, j, k, g, u) = mdc[(u - 1) + 6 * ((m - 1) + (size_t)o.nmat * (g - 1))];
        }
  while (true) {
    Rec r = cr.rec();
    int rot = r.geti();
    if (rot < 1) break;
    while (true) {
      Rec q = cr.rec();
      int x1 = q.geti(), x2 = q.geti(), y1 = q.geti(), y2 = q.geti(), z1 = q.geti(), z2 = q.geti();
      if (x1 < 1 || x2 < 1 || y1 < 1 || y2 < 1 || z1 < 1 || z2 < 1) break;
      if (x1 > o.nx || x2 > o.nx || y1 > o.ny || y2 > o.ny || z1 > o.nz || z2 > o.nz)
        q.fail("wrong position for ADF rotation: out of dimension of the core");
      for (int g = 1; g <= o.ng; ++g)
        for (int k = z1; k <= z2; ++k)
          for (int j = y1; j <= y2; ++j)
            for (int i = x1; i <= x2; ++i) {
              double a1 = XDC(xdc, i, j, k, g, 1), a2 = XDC(xdc, i, j, k, g, 2);
              double a3 = XDC(xdc, i, j, k, g, 3), a4 = XDC(xdc, i, j, k, g, 4);
              double x1v = a1, x2v = a2, x3v = a3, x4v = a4;
              if (rot == 1) { a1 = x4v; a2 = x3v; a3 = x1v; a4 = x2v; }
              if (rot == 2) { a1 = x2v; a2 = x1v; a3 = x4v; a4 = x3v; }
              if (rot == 3) { a1 = x3v; a2 = x4v; a3 = x2v; a4 = x1v; }
              XDC(xdc, i, j, k, g, 1) = a1; XDC(xdc, i, j, k, g, 2) = a2;
              XDC(xdc, i, j, k, g, 3) = a3; XDC(xdc, i, j, k, g, 4) = a4;
            }
    }
  }
  // The optional print line that follows is output only.
  std::vector<int> tx(o.nx + 1), ty(o.ny + 1), tz(o.nz + 1);
  tx[0] = 1; for (int i = 2; i <= o.nx + 1; ++i) tx[i - 1] = tx[i - 2] + o.xdiv[i - 2];
  ty[0] = 1; for (int j = 2; j <= o.ny + 1; ++j) ty[j - 1] = ty[j - 2] + o.ydiv[j - 2];
  tz[0] = 1; for (int k = 2; k <= o.nz + 1; ++k) tz[k - 1] = tz[k - 2] + o.zdiv[k - 2];
  for (int g = 1; g <= o.ng; ++g) {
    int ztot = 0;
    for (int k = 1; k <= o.nz; ++k)
      for (int lz = 1; lz <= o.zdiv[k - 1]; ++lz) {
        ++ztot;
        int ytot = 0;
        for (int j = 1; j <= o.ny; ++j)
          for (int ly = 1; ly <= o.ydiv[j - 1]; ++ly) {
            ++ytot;
            int xtot = 0;
            for (int i = 1; i <= o.nx; ++i)
              for (int lx = 1; lx <= o.xdiv[i - 1]; ++lx) {
                ++xtot;
                int n = o.XYZ(xtot, ytot, ztot);
                if (n == 0) continue;   // only active nodes receive ADFs
                double v[7];
                for (int u = 1; u <= 6; ++u) v[u] = (o.MN(xtot, ytot, ztot) != 0) ? 1.0 : 0.0;
                if (xtot == tx[i - 1]) v[2] = XDC(xdc, i, j, k, g, 2);
                if (xtot == tx[i] - 1) v[1] = XDC(xdc, i, j, k, g, 1);
                if (ytot == ty[j - 1]) v[4] = XDC(xdc, i, j, k, g, 4);
                if (ytot == ty[j] - 1) v[3] = XDC(xdc, i, j, k, g, 3);
                if (ztot == tz[k - 1]) v[5] = XDC(xdc, i, j, k, g, 5);
                if (ztot == tz[k] - 1) v[6] = XDC(xdc, i, j, k, g, 6);
                for (int u = 1; u <= 6; ++u) o.X3(o.dc, n, g, u) = v[u];
              }
          }
      }
  }
}

// Per-material changes of sigtr, siga, nuf, sigf and sigs(g,1..ng): nmat x ng
// records as inp_crod/inp_cbcs/inp_bcon/inp_ftem/inp_mtem/inp_cden read them.
static void read_changes(Ora& o, CardReader& cr, Ora::Feedback& f) {
  const size_t mg = (size_t)o.nmat * o.ng;
  f.str.assign(mg, 0); f.sa = f.nf = f.sf = f.str;
  f.ss.assign(mg * o.ng, 0);
  for (int i = 1; i <= o.nmat; ++i)
    for (int g = 1; g <= o.ng; ++g) {
      Rec x = cr.rec();
      o.M2(f.str, i, g) = x.getd();
      o.M2(f.sa, i, g) = x.getd();
      o.M2(f.nf, i, g) = x.getd();
      o.M2(f.sf, i, g) = x.getd();
      for (int h = 1; h <= o.ng; ++h) o.M3(f.ss, i, g, h) = x.getd();
    }
  f.on = true;
}

// inp_crod (mod_io.f90:2148-2328)
static void read_crod(Ora& o, std::vector<Line>* L) {
  CardReader cr(L, "CROD");
  Rec a = cr.rec();
  o.nb = a.geti();
  o.nstep = a.geti();
  Rec b = cr.rec();
  o.pos0 = b.getd();
  o.ssize = b.getd();
  Rec c = cr.rec();
  o.bpos.assign(o.nb, 0.0);
  for (int i = 0; i < o.nb; ++i) o.bpos[i] = c.getd();
  for (int i = 0; i < o.nb; ++i) {
    if (o.bpos[i] > (double)(float)o.nstep) c.fail("control rod bank position is larger than the number of steps");
    if (o.bpos[i] < 0.) c.fail("control rod bank position is negative");
    if (o.coreh < o.bpos[i] * o.ssize) c.fail("core height is lower than the control rod position");
  }
  std::vector<int> bmap((size_t)o.nx * o.ny);
  for (int j = o.ny; j >= 1; --j) {
    Rec r = cr.rec();
    for (int i = 1; i <= o.nx; ++i) {
      const int v = r.geti();
      if (v > o.nb) r.fail("control rod bank number is larger than the number of banks");
      bmap[(i - 1) + (size_t)o.nx * (j - 1)] = v;
    }
  }
  o.fbmap.assign((size_t)o.nxx * o.nyy, 0);
  int ytot = 0;
  for (int j = 1; j <= o.ny; ++j)
    for (int ly = 1; ly <= o.ydiv[j - 1]; ++ly) {
      ++ytot;
      int xtot = 0;
      for (int i = 1; i <= o.nx; ++i)
        for (int lx = 1; lx <= o.xdiv[i - 1]; ++lx) {
          ++xtot;
          o.fbmap[(xtot - 1) + (size_t)o.nxx * (ytot - 1)] = bmap[(i - 1) + (size_t)o.nx * (j - 1)];
        }
    }
  read_changes(o, cr, o.fb_crod);
}

// inp_ejct (mod_io.f90:2332-2482), without %XTAB: per bank the final
// position, start time and speed; ttot, tstep1, tdiv, tstep2; beta and
// lambda of the six families; the group velocities; an optional print flag
static void read_ejct(Ora& o, std::vector<Line>* L) {
  CardReader cr(L, "EJCT");
  o.fbpos.assign(o.nb, 0.0); o.tmove = o.fbpos; o.bspeed = o.fbpos;
  o.mdir.assign(o.nb, 0);
  for (int i = 0; i < o.nb; ++i) {
    Rec r = cr.rec();
    o.fbpos[i] = r.getd(); o.tmove[i] = r.getd(); o.bspeed[i] = r.getd();
    if (o.fbpos[i] > (double)o.nstep) r.fail("wrong final control rod position");
    if (std::fabs(o.fbpos[i] - o.bpos[i]) < 1.e-5) o.mdir[i] = 0;
    else if (o.fbpos[i] - o.bpos[i] > 1.e-5) o.mdir[i] = 2;
    else o.mdir[i] = 1;
  }
  Rec t = cr.rec();
  o.ttot = t.getd(); o.tstep1 = t.getd(); o.tdiv = t.getd(); o.tstep2 = t.getd();
  Rec b = cr.rec();
  for (int i = 0; i < Ora::nf; ++i) o.ibeta[i] = b.getd();
  Rec l = cr.rec();
  for (int i = 0; i < Ora::nf; ++i) o.lamb[i] = l.getd();
  Rec v = cr.rec();
  o.velo.assign(o.ng, 0.0);
  for (int g = 0; g < o.ng; ++g) o.velo[g] = v.getd();
  if (o.ttot < o.tstep1 || o.ttot < o.tstep2) t.fail("total simulation time shall be greater than the time steps");
  if (o.tdiv < o.tstep1) t.fail("when to start the second time step shall be greater than the first time step");
  if (o.tdiv > o.ttot) t.fail("when to start the second time step shall be less than the total time");
  if (std::lround(o.tdiv / o.tstep1) + std::lround((o.ttot - o.tdiv) / o.tstep2) > 10000)
    t.fail("too many time steps (more than 10000)");
}

// inp_thet (mod_io.f90:1650-1689)
static void read_thet(Ora& o, std::vector<Line>* L) {
  CardReader cr(L, "THET");
  Rec r = cr.rec();
  o.sth = r.getd();
  if (o.sth < 0.001) r.fail("theta value is too small");
  if (o.sth > 1.0) r.fail("theta value shall not greater than 1.0");
  o.bth = (1.0 - o.sth) / o.sth;
}

// inp_cbcs (mod_io.f90:2486-2571) / inp_bcon (:2575-2662) / inp_ftem, inp_mtem,
// inp_cden (:2666-2954): the state value (and reference) then the changes
static void read_state_card(Ora& o, std::vector<Line>* L, const char* name, Ora::Feedback& f, bool has_value) {
  CardReader cr(L, name);
  Rec a = cr.rec();
  if (has_value) {
    f.val = a.getd();
    f.ref = a.getd();
  } else {
    f.ref = a.getd();
    f.val = f.ref;
  }
  read_changes(o, cr, f);
}

static void parse_deck(Ora& o, const std::string& text, const std::string& basedir) {
  std::vector<Line> buf;
  strip_comments(text, buf);
  Cards cards;
  split_cards(buf, basedir, cards);
  static const char* oos[] = {"ESRC", "THER", "XTAB"};
  for (auto& c : cards.cards)
    for (auto k : oos)
      if (c.first == k) throw OraError(ORA_ERR_UNSUPPORTED, "card %" + c.first + " is outside the static k-eigenvalue path");
  auto* m = cards.find("MODE");
  if (!m || m->empty()) throw OraError(ORA_ERR_INPUT, "card %MODE does not present. this card is mandatory");
  o.mode = upper(trim((*m)[0].text));
  if (o.mode != "FORWARD" && o.mode != "ADJOINT" && o.mode != "BCSEARCH" && o.mode != "RODEJECT") {
    if (o.mode == "FIXEDSRC")
      throw OraError(ORA_ERR_UNSUPPORTED, "mode " + o.mode + " is outside the static k-eigenvalue path");
    throw OraError(ORA_ERR_INPUT, "mode " + o.mode + " is unidentified");
  }
  if (auto* k = cards.find("KERN")) read_kern(o, k);
  auto* x = cards.find("XSEC");
  if (!x) throw OraError(ORA_ERR_INPUT, "card %XSEC or %XTAB does not present. this card is mandatory");
  read_xsec(o, x);
  auto* g = cards.find("GEOM");
  if (!g) throw OraError(ORA_ERR_INPUT, "card %GEOM does not present. this card is mandatory");
  read_geom(o, g);
  if (auto* p = cards.find("PRNT")) {
    CardReader cr(p, "PRNT");
    Rec r = cr.rec();
    o.aprad = r.geti(); o.apaxi = r.geti(); o.afrad = r.geti();
  }
  misc(o);
  o.coreh = 0.0;
  for (int k = 0; k < o.nzz; ++k) o.coreh = o.coreh + o.zdel[k];
  if (auto* c = cards.find("CROD")) read_crod(o, c);
  if (auto* c = cards.find("CBCS")) { read_state_card(o, c, "CBCS", o.fb_bcon, false); o.bcbcs = true; }
  else if (auto* c = cards.find("BCON")) { read_state_card(o, c, "BCON", o.fb_bcon, true); o.bcon = o.fb_bcon.val; }
  if (auto* c = cards.find("FTEM")) read_state_card(o, c, "FTEM", o.fb_ftem, true);
  if (auto* c = cards.find("MTEM")) read_state_card(o, c, "MTEM", o.fb_mtem, true);
  if (auto* c = cards.find("CDEN")) read_state_card(o, c, "CDEN", o.fb_cden, true);
  // card checks of mode BCSEARCH (mod_io.f90:196-214)
  if (o.mode == "BCSEARCH" && !o.bcbcs)
    throw OraError(ORA_ERR_INPUT, "mode BCSEARCH needs card %CBCS");
  if (o.mode != "BCSEARCH" && o.bcbcs)
    throw OraError(ORA_ERR_INPUT, "card %CBCS is not necessary for this calculation mode");
  if (o.mode == "BCSEARCH" && cards.find("BCON"))
    throw OraError(ORA_ERR_INPUT, "card %BCON must not present for this calculation mode");
  // card checks of mode RODEJECT (mod_io.f90:227-245)
  auto* ej = cards.find("EJCT");
  if (o.mode == "RODEJECT" && !ej) throw OraError(ORA_ERR_INPUT, "mode RODEJECT needs card %EJCT");
  if (o.mode == "RODEJECT" && !cards.find("CROD")) throw OraError(ORA_ERR_INPUT, "mode RODEJECT needs card %CROD");
  if (o.mode != "RODEJECT" && ej) throw OraError(ORA_ERR_INPUT, "card %EJCT is not necessary for this calculation mode");
  if (ej) read_ejct(o, ej);
  if (auto* it = cards.find("ITER")) read_iter(o, it);
  if (auto* th = cards.find("THET")) read_thet(o, th);
  o.bextr = cards.find("EXTR") != nullptr;
  o.dc.assign((size_t)o.nnod * o.ng * 6, 1.0);
  if (auto* a = cards.find("ADF")) { o.badf = true; read_adf(o, a); }
  o.exsrc.assign((size_t)o.nnod * o.ng, 0.0);
}

// ===========================================================================
// Cross sections (mod_xsec.f90)
// ===========================================================================

// base_updt (mod_xsec.f90:172-195)
static void base_updt(Ora& o) {
  for (int n = 1; n <= o.nnod; ++n) {
    int m = o.mat[n - 1];
    for (int g = 1; g <= o.ng; ++g) {
      o.N2(o.sigtr, n, g) = o.M2(o.xsigtr, m, g);
      o.N2(o.siga, n, g) = o.M2(o.xsiga, m, g);
      o.N2(o.nuf, n, g) = o.M2(o.xnuf, m, g);
      o.N2(o.sigf, n, g) = o.M2(o.xsigf, m, g);
      for (int h = 1; h <= o.ng; ++h) o.SG(o.sigs, n, g, h) = o.M3(o.xsigs, m, g, h);
    }
  }
}

// Dsigr_updt (mod_xsec.f90:199-226)
static void dsigr_updt(Ora& o) {
  for (int i = 1; i <= o.nnod; ++i)
    for (int g = 1; g <= o.ng; ++g) {
      if (o.N2(o.sigtr, i, g) < F_1em5) throw OraError(ORA_ERR_BADXS, "negative diffusion coefficient encountered");
      o.N2(o.D, i, g) = 1.0 / (3.0 * o.N2(o.sigtr, i, g));
      double dum = 0.;
      for (int h = 1; h <= o.ng; ++h) if (g != h) dum = dum + o.SG(o.sigs, i, g, h);
      o.N2(o.sigr, i, g) = o.N2(o.siga, i, g) + dum;
    }
}

// check_xs (mod_xsec.f90:90-168)
static void check_xs(Ora& o) {
  for (int g = 1; g <= o.ng; ++g) {
    for (int n = 1; n <= o.nnod; ++n) {
      if (o.N2(o.D, n, g) < F_1em20) throw OraError(ORA_ERR_BADXS, "diffusion coef. is close to zero or negative");
      if (o.N2(o.sigr, n, g) < 0.) throw OraError(ORA_ERR_BADXS, "removal xs is negative");
      if (o.N2(o.nuf, n, g) < 0.) throw OraError(ORA_ERR_BADXS, "nu*fission xs is negative");
    }
    for (int n = 1; n <= o.nmat; ++n)
      if (o.M2(o.chi, n, g) < 0.) throw OraError(ORA_ERR_BADXS, "fission spectrum is negative");
    for (int h = 1; h <= o.ng; ++h)
      for (int n = 1; n <= o.nnod; ++n)
        if (o.SG(o.sigs, n, g, h) < 0.) throw OraError(ORA_ERR_BADXS, "scattering xs is negative");
  }
}

// bcon_updt / ftem_updt / mtem_updt / cden_updt (mod_xsec.f90:394-521):
// node XS += change(mat) * dv, dv the state's difference from its reference
// (sqrt(T) - sqrt(Tref) for the fuel temperature)
static void state_updt(Ora& o, const Ora::Feedback& f, double dv) {
  for (int n = 1; n <= o.nnod; ++n) {
    const int m = o.mat[n - 1];
    for (int g = 1; g <= o.ng; ++g) {
      o.N2(o.sigtr, n, g) = o.N2(o.sigtr, n, g) + o.M2(const_cast<std::vector<double>&>(f.str), m, g) * dv;
      o.N2(o.siga, n, g) = o.N2(o.siga, n, g) + o.M2(const_cast<std::vector<double>&>(f.sa), m, g) * dv;
      o.N2(o.nuf, n, g) = o.N2(o.nuf, n, g) + o.M2(const_cast<std::vector<double>&>(f.nf), m, g) * dv;
      o.N2(o.sigf, n, g) = o.N2(o.sigf, n, g) + o.M2(const_cast<std::vector<double>&>(f.sf), m, g) * dv;
      for (int h = 1; h <= o.ng; ++h)
        o.SG(o.sigs, n, g, h) = o.SG(o.sigs, n, g, h) + o.M3(const_cast<std::vector<double>&>(f.ss), m, g, h) * dv;
    }
  }
}

// crod_updt (mod_xsec.f90:230-303): fully rodded nodes get the rod changes,
// the node holding the rod tip a volume fraction of them; then negative
// siga, nuf, sigf and sigs of the rodded columns are set to zero
static void crod_updt(Ora& o) {
  const Ora::Feedback& f = o.fb_crod;
  auto add = [&](int n, double w) {
    const int m = o.mat[n - 1];
    for (int g = 1; g <= o.ng; ++g) {
      o.N2(o.sigtr, n, g) = o.N2(o.sigtr, n, g) + w * o.M2(const_cast<std::vector<double>&>(f.str), m, g);
      o.N2(o.siga, n, g) = o.N2(o.siga, n, g) + w * o.M2(const_cast<std::vector<double>&>(f.sa), m, g);
      o.N2(o.nuf, n, g) = o.N2(o.nuf, n, g) + w * o.M2(const_cast<std::vector<double>&>(f.nf), m, g);
      o.N2(o.sigf, n, g) = o.N2(o.sigf, n, g) + w * o.M2(const_cast<std::vector<double>&>(f.sf), m, g);
      for (int h = 1; h <= o.ng; ++h)
        o.SG(o.sigs, n, g, h) = o.SG(o.sigs, n, g, h) + w * o.M3(const_cast<std::vector<double>&>(f.ss), m, g, h);
    }
  };
  auto addfull = [&](int n) {   // the reference adds the change itself (no factor) to fully rodded nodes
    const int m = o.mat[n - 1];
    for (int g = 1; g <= o.ng; ++g) {
      o.N2(o.sigtr, n, g) = o.N2(o.sigtr, n, g) + o.M2(const_cast<std::vector<double>&>(f.str), m, g);
      o.N2(o.siga, n, g) = o.N2(o.siga, n, g) + o.M2(const_cast<std::vector<double>&>(f.sa), m, g);
      o.N2(o.nuf, n, g) = o.N2(o.nuf, n, g) + o.M2(const_cast<std::vector<double>&>(f.nf), m, g);
      o.N2(o.sigf, n, g) = o.N2(o.sigf, n, g) + o.M2(const_cast<std::vector<double>&>(f.sf), m, g);
      for (int h = 1; h <= o.ng; ++h)
        o.SG(o.sigs, n, g, h) = o.SG(o.sigs, n, g, h) + o.M3(const_cast<std::vector<double>&>(f.ss), m, g, h);
    }
  };
  for (int j = 1; j <= o.nyy; ++j)
    for (int i = 1; i <= o.nxx; ++i) {
      const int bank = o.fbmap[(i - 1) + (size_t)o.nxx * (j - 1)];
      if (bank <= 0) continue;
      const double rodh = o.coreh - o.pos0 - o.bpos[bank - 1] * o.ssize;
      double dum = 0.0;
      for (int k = o.nzz; k >= 1; --k) {
        const int n = o.XYZ(i, j, k);
        if (rodh >= dum && rodh <= dum + o.zdel[k - 1]) {
          const double vfrac = (rodh - dum) / o.zdel[k - 1];
          if (n > 0) add(n, vfrac);
          break;
        }
        if (n > 0) addfull(n);
        dum = dum + o.zdel[k - 1];
      }
      for (int k = o.nzz; k >= 1; --k) {
        const int n = o.XYZ(i, j, k);
        if (n <= 0) continue;
        for (int g = 1; g <= o.ng; ++g) {
          if (o.N2(o.siga, n, g) < 0.) o.N2(o.siga, n, g) = 0.;
          if (o.N2(o.nuf, n, g) < 0.) o.N2(o.nuf, n, g) = 0.;
          if (o.N2(o.sigf, n, g) < 0.) o.N2(o.sigf, n, g) = 0.;
          for (int h = 1; h <= o.ng; ++h)
            if (o.SG(o.sigs, n, g, h) < 0.) o.SG(o.sigs, n, g, h) = 0.;
        }
      }
    }
}

// XS_updt (mod_xsec.f90:11-46): base, the feedback updates in the
// reference's order (boron, fuel temperature, moderator temperature,
// coolant density, control rods), D/sigr and the checks.  xbcon is the
// boron concentration (cbsearch passes its iterate).
static void xs_updt_at(Ora& o, double xbcon) {
  base_updt(o);
  if (o.fb_bcon.on) state_updt(o, o.fb_bcon, xbcon - o.fb_bcon.ref);
  if (o.fb_ftem.on) state_updt(o, o.fb_ftem, std::sqrt(o.fb_ftem.val) - std::sqrt(o.fb_ftem.ref));
  if (o.fb_mtem.on) state_updt(o, o.fb_mtem, o.fb_mtem.val - o.fb_mtem.ref);
  if (o.fb_cden.on) state_updt(o, o.fb_cden, o.fb_cden.val - o.fb_cden.ref);
  if (o.fb_crod.on) crod_updt(o);
  dsigr_updt(o);
  check_xs(o);
}

static void xs_updt(Ora& o) { xs_updt_at(o, o.bcon); }

// ===========================================================================
// CMFD (mod_cmfd.f90)
// ===========================================================================

// coup_coef (mod_cmfd.f90:11-137)
static void coup_coef(Ora& o) {
  const double alb = 1.e30;
  if (o.coup_first) {
    o.df.assign((size_t)o.nnod * o.ng * 6, 0.0);
    o.dn.assign((size_t)o.nnod * o.ng * 6, 0.0);
    o.coup_first = false;
  }
  auto bnd = [&](int bc, double Dn, double h) -> double {
    if (bc == 0) return 2.0 * alb * Dn / (2.0 * Dn + alb * h);
    if (bc == 1) return Dn / (2.0 * Dn + 0.5 * h);
    return 0.0;
  };
  for (int g = 1; g <= o.ng; ++g)
    for (int n = 1; n <= o.nnod; ++n) {
      int i = o.ix[n - 1], j = o.iy[n - 1], k = o.iz[n - 1];
      double Dn = o.N2(o.D, n, g);
      if (i == o.ysmax[j - 1]) o.X3(o.df, n, g, 1) = bnd(o.xeast, Dn, o.xdel[i - 1]);
      else {
        double d2 = o.N2(o.D, o.XYZ(i + 1, j, k), g);
        o.X3(o.df, n, g, 1) = 2.0 * Dn * d2 / (Dn * o.xdel[i] + d2 * o.xdel[i - 1]);
      }
      if (i == o.ysmin[j - 1]) o.X3(o.df, n, g, 2) = bnd(o.xwest, Dn, o.xdel[i - 1]);
      else {
        double d1 = o.N2(o.D, o.XYZ(i - 1, j, k), g);
        o.X3(o.df, n, g, 2) = 2.0 * Dn * d1 / (Dn * o.xdel[i - 2] + d1 * o.xdel[i - 1]);
      }
      if (j == o.xsmax[i - 1]) o.X3(o.df, n, g, 3) = bnd(o.ynorth, Dn, o.ydel[j - 1]);
      else {
        double d2 = o.N2(o.D, o.XYZ(i, j + 1, k), g);
        o.X3(o.df, n, g, 3) = 2.0 * Dn * d2 / (Dn * o.ydel[j] + d2 * o.ydel[j - 1]);
      }
      if (j == o.xsmin[i - 1]) o.X3(o.df, n, g, 4) = bnd(o.ysouth, Dn, o.ydel[j - 1]);
      else {
        double d1 = o.N2(o.D, o.XYZ(i, j - 1, k), g);
        o.X3(o.df, n, g, 4) = 2.0 * Dn * d1 / (Dn * o.ydel[j - 2] + d1 * o.ydel[j - 1]);
      }
      if (k == o.nzz) o.X3(o.df, n, g, 5) = bnd(o.ztop, Dn, o.zdel[k - 1]);
      else {
        double d2 = o.N2(o.D, o.XYZ(i, j, k + 1), g);
        o.X3(o.df, n, g, 5) = 2.0 * Dn * d2 / (Dn * o.zdel[k] + d2 * o.zdel[k - 1]);
      }
      if (k == 1) o.X3(o.df, n, g, 6) = bnd(o.zbott, Dn, o.zdel[k - 1]);
      else {
        double d1 = o.N2(o.D, o.XYZ(i, j, k - 1), g);
        o.X3(o.df, n, g, 6) = 2.0 * Dn * d1 / (Dn * o.zdel[k - 2] + d1 * o.zdel[k - 1]);
      }
    }
}

// set_ind (mod_cmfd.f90:141-213)
static void set_ind(Ora& o) {
  std::vector<int> nodp((size_t)o.nxx * o.nyy, 0);
  auto NP = [&](int i, int j) -> int& { return nodp[(i - 1) + (size_t)o.nxx * (j - 1)]; };
  int rec = 0;
  for (int j = 1; j <= o.nyy; ++j)
    for (int i = o.ysmin[j - 1]; i <= o.ysmax[j - 1]; ++i) { ++rec; NP(i, j) = rec; }
  int np = rec;
  for (int n = 1; n <= o.nnod; ++n) {
    int i = o.ix[n - 1], j = o.iy[n - 1], k = o.iz[n - 1];
    rec = 0;
    if (k != 1) o.COL(n, ++rec) = n - np;
    if (j != o.xsmin[i - 1]) o.COL(n, ++rec) = n - (NP(i, j) - NP(i, j - 1));
    if (i != o.ysmin[j - 1]) o.COL(n, ++rec) = n - 1;
    o.COL(n, ++rec) = n;
    if (i != o.ysmax[j - 1]) o.COL(n, ++rec) = n + 1;
    if (j != o.xsmax[i - 1]) o.COL(n, ++rec) = n + (NP(i, j + 1) - NP(i, j));
    if (k != o.nzz) o.COL(n, ++rec) = n + np;
  }
}

// matrix_setup (mod_cmfd.f90:217-304)
static void matrix_setup(Ora& o, int opt) {
  if (o.matrix_first) {
    o.Amat.assign((size_t)7 * o.nnod * o.ng, 0.0);
    set_ind(o);
    o.matrix_first = false;
  }
  if (opt > 0) coup_coef(o);
  for (int g = 1; g <= o.ng; ++g)
    for (int n = 1; n <= o.nnod; ++n) {
      int i = o.ix[n - 1], j = o.iy[n - 1], k = o.iz[n - 1];
      double xd = o.xdel[i - 1], yd = o.ydel[j - 1], zd = o.zdel[k - 1];
      auto DF = [&](int u) { return o.X3(o.df, n, g, u); };
      auto DN = [&](int u) { return o.X3(o.dn, n, g, u); };
      int rec = 0;
      if (k != 1) o.AE(++rec, n, g) = -(DF(6) - DN(6)) / zd;
      if (j != o.xsmin[i - 1]) o.AE(++rec, n, g) = -(DF(4) - DN(4)) / yd;
      if (i != o.ysmin[j - 1]) o.AE(++rec, n, g) = -(DF(2) - DN(2)) / xd;
      o.AE(++rec, n, g) = (DF(1) + DF(2) - DN(1) + DN(2)) / xd +
                          (DF(3) + DF(4) - DN(3) + DN(4)) / yd +
                          (DF(5) + DF(6) - DN(5) + DN(6)) / zd + o.N2(o.sigr, n, g);
      if (i != o.ysmax[j - 1]) o.AE(++rec, n, g) = -(DF(1) + DN(1)) / xd;
      if (j != o.xsmax[i - 1]) o.AE(++rec, n, g) = -(DF(3) + DN(3)) / yd;
      if (k != o.nzz) o.AE(++rec, n, g) = -(DF(5) + DN(5)) / zd;
    }
}

// sp_matvec (mod_cmfd.f90:1247-1268)
static void sp_matvec(Ora& o, int g, const double* x, double* v) {
  for (int n = 1; n <= o.nnod; ++n) {
    double s = 0.0;
    for (int i = 1; i <= o.ncol[n - 1]; ++i) s = s + o.AE(i, n, g) * x[o.COL(n, i) - 1];
    v[n - 1] = s;
  }
}

// dproduct (mod_cmfd.f90:1272-1286)
static double dproduct(const std::vector<double>& a, const std::vector<double>& b) {
  double x = 0.0;
  for (size_t n = 0; n < a.size(); ++n) x = x + a[n] * b[n];
  return x;
}

// bicg (mod_cmfd.f90:1203-1243): exactly imax unpreconditioned BiCGSTAB steps
static void bicg(Ora& o, int imax, int g, const std::vector<double>& b, double* x) {
  int N = o.nnod;
  std::vector<double> r(N), rs(N), v(N, 0.0), p(N, 0.0), s(N), t(N), tmp(N);
  sp_matvec(o, g, x, tmp.data());
  for (int n = 0; n < N; ++n) r[n] = b[n] - tmp[n];
  rs = r;
  double rho = 1.0, alpha = 1.0, omega = 1.0, rho_prev, beta, theta;
#ifdef ORA_RHO_FROM_S_T
  // Sensitivity build only: (rs, r) of the next step formed as
  // (rs,s) - omega (rs,t), algebraically equal to dproduct(rs, r) of
  // mod_cmfd.f90:1230, the way the CUDA path evaluates it.
  double rho_next = dproduct(rs, r);
#endif
  for (int i = 1; i <= imax; ++i) {
    rho_prev = rho;
#ifdef ORA_RHO_FROM_S_T
    rho = rho_next;
#else
    rho = dproduct(rs, r);
#endif
    beta = (rho / rho_prev) * (alpha / omega);
    for (int n = 0; n < N; ++n) p[n] = r[n] + beta * (p[n] - omega * v[n]);
    sp_matvec(o, g, p.data(), v.data());
    alpha = rho / dproduct(rs, v);
    for (int n = 0; n < N; ++n) s[n] = r[n] - alpha * v[n];
    sp_matvec(o, g, s.data(), t.data());
    theta = dproduct(t, t);
    omega = dproduct(t, s) / theta;
#ifdef ORA_RHO_FROM_S_T
    rho_next = dproduct(rs, s) - omega * dproduct(rs, t);
#endif
    for (int n = 0; n < N; ++n) x[n] = x[n] + alpha * p[n] + omega * s[n];
    for (int n = 0; n < N; ++n) r[n] = s[n] - omega * t[n];
  }
}

// FSrc (mod_cmfd.f90:956-977) / FSrcAd (mod_cmfd.f90:981-1002)
static void fsrc(Ora& o, std::vector<double>& fs, bool adj) {
  std::fill(fs.begin(), fs.end(), 0.0);
  for (int g = 1; g <= o.ng; ++g)
    for (int n = 1; n <= o.nnod; ++n) {
      double w = adj ? o.M2(o.chi, o.mat[n - 1], g) : o.N2(o.nuf, n, g);
      fs[n - 1] = fs[n - 1] + o.N2(o.f0, n, g) * w;
    }
}

// TSrc (mod_cmfd.f90:1006-1033) / TSrcAd (mod_cmfd.f90:1037-1064)
static void tsrc(Ora& o, int g, double Keff, std::vector<double>& bs, bool adj) {
  std::fill(o.s0.begin(), o.s0.end(), 0.0);
  for (int h = 1; h <= o.ng; ++h)
    for (int n = 1; n <= o.nnod; ++n)
      if (g != h) {
        double sg = adj ? o.SG(o.sigs, n, g, h) : o.SG(o.sigs, n, h, g);
        o.N2(o.s0, n, g) = o.N2(o.s0, n, g) + sg * o.N2(o.f0, n, h);
      }
  for (int n = 1; n <= o.nnod; ++n) {
    double w = adj ? o.N2(o.nuf, n, g) : o.M2(o.chi, o.mat[n - 1], g);
    bs[n - 1] = w * o.fs0[n - 1] / Keff + o.N2(o.s0, n, g) + o.N2(o.exsrc, n, g);
  }
}

// l2norm (mod_cmfd.f90:1100-1116)
static double l2norm(const std::vector<double>& a) {
  double x = 0.0;
  for (double v : a) x = x + v * v;
  return std::sqrt(x);
}

// Integrate (mod_cmfd.f90:1120-1139)
static double integrate(Ora& o, const std::vector<double>& s) {
  double intg = 0.;
  for (int n = 1; n <= o.nnod; ++n) intg = intg + o.vdel[n - 1] * s[n - 1];
  return intg;
}

// RelE (mod_cmfd.f90:1143-1168)
static double rele(Ora& o, const std::vector<double>& nw, const std::vector<double>& old) {
  double rel = 0.;
  for (int n = 1; n <= o.nnod; ++n)
    if (std::fabs(nw[n - 1]) > 1.e-10) {
      double e = std::fabs(nw[n - 1] - old[n - 1]) / std::fabs(nw[n - 1]);
      if (e > rel) rel = e;
    }
  return rel;
}

// RelEg (mod_cmfd.f90:1172-1199)
static double releg(Ora& o, const std::vector<double>& nw, const std::vector<double>& old) {
  double rel = 0.;
  for (int n = 1; n <= o.nnod; ++n)
    for (int g = 1; g <= o.ng; ++g) {
      size_t q = (n - 1) + (size_t)o.nnod * (g - 1);
      if (std::fabs(nw[q]) > 1.e-10) {
        double e = std::fabs(nw[q] - old[q]) / std::fabs(nw[q]);
        if (e > rel) rel = e;
      }
    }
  return rel;
}

// fiss_extrp (mod_cmfd.f90:308-335); the sign test at :328 never fires.
static void fiss_extrp(double e1, double e2, const std::vector<double>& errn, std::vector<double>& fs) {
  double domiR = e2 / e1;
  double c = domiR / (1.0 - domiR);
  for (size_t n = 0; n < fs.size(); ++n) fs[n] = fs[n] + c * errn[n];
}

// ===========================================================================
// Nodal (mod_nodal.f90)
// ===========================================================================

static inline double hdir(Ora& o, int u, int n) {
  if (u == 1) return o.xdel[o.ix[n - 1] - 1];
  if (u == 2) return o.ydel[o.iy[n - 1] - 1];
  return o.zdel[o.iz[n - 1] - 1];
}

// get_B (mod_nodal.f90:1345-1405); cmode 1 forward, 0 adjoint
static void get_B(Ora& o, int u, int n, std::vector<double>& B) {
  double dn = hdir(o, u, n);
  int m = o.mat[n - 1];
  for (int g = 1; g <= o.ng; ++g)
    for (int h = 1; h <= o.ng; ++h) {
      double dum;
      if (o.cmode == 2) {
        // transient (mod_nodal.f90:1379-1390): prompt and delayed fission of
        // the step, no eigenvalue; the diagonal carries chi twice, as the
        // reference writes it
        const double w = (1.0 - o.tbeta[m - 1] + o.dfis[n - 1]);
        if (g == h) dum = o.N2(o.sigr, n, g) - w * o.M2(o.chi, m, g) * o.M2(o.chi, m, g) * o.N2(o.nuf, n, h);
        else dum = -o.SG(o.sigs, n, h, g) - w * o.M2(o.chi, m, g) * o.N2(o.nuf, n, h);
      } else if (g == h) dum = o.N2(o.sigr, n, g) - o.M2(o.chi, m, g) * o.N2(o.nuf, n, h) / o.Ke;
      else if (o.cmode == 1) dum = -o.SG(o.sigs, n, h, g) - o.M2(o.chi, m, g) * o.N2(o.nuf, n, h) / o.Ke;
      else dum = -o.SG(o.sigs, n, g, h) - o.M2(o.chi, m, h) * o.N2(o.nuf, n, g) / o.Ke;
      o.Bm(B, g, h) = 0.25 * (dn * dn) / o.N2(o.D, n, g) * dum;
    }
}

// get_ABEFGH (mod_nodal.f90:1409-1451)
static void get_ABEFGH(Ora& o, int n, int u, std::vector<double>& Aa, std::vector<double>& Bb, std::vector<double>& Ee,
                       std::vector<double>& Ff, std::vector<double>& Gg, std::vector<double>& Hh) {
  double dn = hdir(o, u, n);
  for (int g = 1; g <= o.ng; ++g) {
    double alp = 0.5 * std::sqrt(o.N2(o.sigr, n, g) / o.N2(o.D, n, g)) * dn;
    double alp2 = alp * alp;
    double sh = std::sinh(alp), ch = std::cosh(alp);
    double m0c = sh / alp;
    double m1s = 3.0 * (ch / alp - sh / alp2);
    double m2c = 5.0 * (sh / alp - 3.0 * ch / alp2 + 3.0 * sh / (alp * alp * alp));
    Aa[g - 1] = (sh - m1s) / (alp2 * m1s);
    Bb[g - 1] = (ch - m0c - m2c) / (alp2 * m2c);
    Ee[g - 1] = (m0c / m2c - 3.0 / alp2);
    Ff[g - 1] = (alp * ch - m1s) / (alp2 * m1s);
    Gg[g - 1] = (alp * sh - 3.0 * m2c) / (ch - m0c - m2c);
    Hh[g - 1] = (alp * ch - m1s) / (sh - m1s);
  }
}

// Lxyz (mod_nodal.f90:901-1005)
static void lxyz(Ora& o, int n, int g, double& L1, double& L2, double& L3) {
  int i = o.ix[n - 1], j = o.iy[n - 1], k = o.iz[n - 1];
  auto DF = [&](int u) { return o.X3(o.df, n, g, u); };
  auto DN = [&](int u) { return o.X3(o.dn, n, g, u); };
  auto F = [&](int m) { return o.N2(o.f0, m, g); };
  double fn = F(n), jp, jm;
  int p = 0, m = 0;
  if (i != o.ysmax[j - 1]) p = o.XYZ(i + 1, j, k);
  if (i != o.ysmin[j - 1]) m = o.XYZ(i - 1, j, k);
  if (i == o.ysmax[j - 1]) jp = (o.xeast == 2) ? 0.0 : DF(1) * fn - DN(1) * fn;
  else jp = -DF(1) * (F(p) - fn) - DN(1) * (F(p) + fn);
  if (i == o.ysmin[j - 1]) jm = (o.xwest == 2) ? 0.0 : -DF(2) * fn - DN(2) * fn;
  else jm = -DF(2) * (fn - F(m)) - DN(2) * (fn + F(m));
  L1 = (jp - jm) / o.xdel[i - 1];
  if (j != o.xsmax[i - 1]) p = o.XYZ(i, j + 1, k);
  if (j != o.xsmin[i - 1]) m = o.XYZ(i, j - 1, k);
  if (j == o.xsmax[i - 1]) jp = (o.ynorth == 2) ? 0.0 : DF(3) * fn - DN(3) * fn;
  else jp = -DF(3) * (F(p) - fn) - DN(3) * (F(p) + fn);
  if (j == o.xsmin[i - 1]) jm = (o.ysouth == 2) ? 0.0 : -DF(4) * fn - DN(4) * fn;
  else jm = -DF(4) * (fn - F(m)) - DN(4) * (fn + F(m));
  L2 = (jp - jm) / o.ydel[j - 1];
  if (k != o.nzz) p = o.XYZ(i, j, k + 1);
  if (k != 1) m = o.XYZ(i, j, k - 1);
  if (k == o.nzz) jp = (o.ztop == 2) ? 0.0 : DF(5) * fn - DN(5) * fn;
  else jp = -DF(5) * (F(p) - fn) - DN(5) * (F(p) + fn);
  if (k == 1) jm = (o.zbott == 2) ? 0.0 : -DF(6) * fn - DN(6) * fn;
  else jm = -DF(6) * (fn - F(m)) - DN(6) * (fn + F(m));
  L3 = (jp - jm) / o.zdel[k - 1];
}

// get_source (mod_nodal.f90:1009-1043)
static void get_source(Ora& o) {
  if (o.source_first) {
    o.S1.assign((size_t)o.nnod * o.ng, 0); o.S2 = o.S1; o.S3 = o.S1;
    o.source_first = false;
  }
  for (int g = 1; g <= o.ng; ++g)
    for (int n = 1; n <= o.nnod; ++n) {
      double L1, L2, L3;
      lxyz(o, n, g, L1, L2, L3);
      if (o.cmode == 2) {   // transient: the step's external source joins the leakage (:1031-1035)
        o.N2(o.S1, n, g) = L2 + L3 - o.N2(o.exsrc, n, g);
        o.N2(o.S2, n, g) = L1 + L3 - o.N2(o.exsrc, n, g);
        o.N2(o.S3, n, g) = L1 + L2 - o.N2(o.exsrc, n, g);
      } else {
        o.N2(o.S1, n, g) = L2 + L3;
        o.N2(o.S2, n, g) = L1 + L3;
        o.N2(o.S3, n, g) = L1 + L2;
      }
    }
}

// Shared helper for TLUpd1/TLUpd2: line geometry of node n in direction u.
struct LineInfo {
  int pos;        // 0 = first node, 2 = last node, 1 = interior
  bool refl;      // reflective at the side that is open (first: minus side, last: plus side)
  int p, m;       // neighbour node numbers (0 when absent)
  double hm, h0, hp;
  std::vector<double>* S;
};

static LineInfo line_info(Ora& o, int u, int n) {
  LineInfo L{};
  int i = o.ix[n - 1], j = o.iy[n - 1], k = o.iz[n - 1];
  if (u == 1) {
    if (i != o.ysmax[j - 1]) L.p = o.XYZ(i + 1, j, k);
    if (i != o.ysmin[j - 1]) L.m = o.XYZ(i - 1, j, k);
    L.h0 = o.xdel[i - 1];
    if (L.p) L.hp = o.xdel[i];
    if (L.m) L.hm = o.xdel[i - 2];
    if (i == o.ysmin[j - 1]) { L.pos = 0; L.refl = (o.xwest == 2); }
    else if (i == o.ysmax[j - 1]) { L.pos = 2; L.refl = (o.xeast == 2); }
    else L.pos = 1;
    L.S = &o.S1;
  } else if (u == 2) {
    if (j != o.xsmax[i - 1]) L.p = o.XYZ(i, j + 1, k);
    if (j != o.xsmin[i - 1]) L.m = o.XYZ(i, j - 1, k);
    L.h0 = o.ydel[j - 1];
    if (L.p) L.hp = o.ydel[j];
    if (L.m) L.hm = o.ydel[j - 2];
    if (j == o.xsmin[i - 1]) { L.pos = 0; L.refl = (o.ysouth == 2); }
    else if (j == o.xsmax[i - 1]) { L.pos = 2; L.refl = (o.ynorth == 2); }
    else L.pos = 1;
    L.S = &o.S2;
  } else {
    if (k != o.nzz) L.p = o.XYZ(i, j, k + 1);
    if (k != 1) L.m = o.XYZ(i, j, k - 1);
    L.h0 = o.zdel[k - 1];
    if (L.p) L.hp = o.zdel[k];
    if (L.m) L.hm = o.zdel[k - 2];
    if (k == 1) { L.pos = 0; L.refl = (o.zbott == 2); }
    else if (k == o.nzz) { L.pos = 2; L.refl = (o.ztop == 2); }
    else L.pos = 1;
    L.S = &o.S3;
  }
  return L;
}

// TLUpd1 (mod_nodal.f90:1047-1199)
static double tlupd1(Ora& o, int u, int n, int g) {
  LineInfo L = line_info(o, u, n);
  auto S = [&](int q) { return o.N2(*L.S, q, g); };
  double Lmom1, tm, tp, p1m, p2m, p1p, p2p, hp;
  if (L.pos == 0) {
    if (L.refl) {
      tm = 1.0; tp = L.hp / L.h0;
      p1m = tm + 1.0; p2m = 2.0 * tm + 1.0;
      p1p = tp + 1.0;
      hp = 2.0 * p1m * p1p * (tm + tp + 1.0);
      Lmom1 = (p1m * p2m * (S(L.p) - S(n))) / hp;
    } else {
      tp = L.hp / L.h0;
      p1p = tp + 1.0;
      Lmom1 = (S(L.p) - S(n)) / p1p;
    }
  } else if (L.pos == 2) {
    if (L.refl) {
      tm = L.hm / L.h0; tp = 1.0;
      p1m = tm + 1.0;
      p1p = tp + 1.0; p2p = 2.0 * tp + 1.0;
      hp = 2.0 * p1m * p1p * (tm + tp + 1.0);
      Lmom1 = (p1p * p2p * (S(n) - S(L.m))) / hp;
    } else {
      tm = L.hm / L.h0;
      p1m = tm + 1.0;
      Lmom1 = (S(n) - S(L.m)) / p1m;
    }
  } else {
    tm = L.hm / L.h0; tp = L.hp / L.h0;
    p1m = tm + 1.0; p2m = 2.0 * tm + 1.0;
    p1p = tp + 1.0; p2p = 2.0 * tp + 1.0;
    hp = 2.0 * p1m * p1p * (tm + tp + 1.0);
    Lmom1 = (p1m * p2m * (S(L.p) - S(n)) + p1p * p2p * (S(n) - S(L.m))) / hp;
  }
  return 0.25 * (L.h0 * L.h0) / o.N2(o.D, n, g) * Lmom1;
}

// TLUpd2 (mod_nodal.f90:1203-1341)
static double tlupd2(Ora& o, int u, int n, int g) {
  LineInfo L = line_info(o, u, n);
  auto S = [&](int q) { return o.N2(*L.S, q, g); };
  double Lmom2, tm, tp, p1m, p1p, hp;
  if (L.pos == 0) {
    if (L.refl) {
      tm = 1.0; tp = L.hp / L.h0;
      p1m = tm + 1.0; p1p = tp + 1.0;
      hp = 2.0 * p1m * p1p * (tm + tp + 1.0);
      Lmom2 = (p1m * (S(L.p) - S(n))) / hp;
    } else {
      Lmom2 = 0.0;
    }
  } else if (L.pos == 2) {
    if (L.refl) {
      tm = L.hm / L.h0; tp = 1.0;
      p1m = tm + 1.0; p1p = tp + 1.0;
      hp = 2.0 * p1m * p1p * (tm + tp + 1.0);
      Lmom2 = (p1p * (S(L.m) - S(n))) / hp;
    } else {
      Lmom2 = 0.0;
    }
  } else {
    tm = L.hm / L.h0; tp = L.hp / L.h0;
    p1m = tm + 1.0; p1p = tp + 1.0;
    hp = 2.0 * p1m * p1p * (tm + tp + 1.0);
    Lmom2 = (p1m * (S(L.p) - S(n)) + p1p * (S(L.m) - S(n))) / hp;
  }
  return 0.25 * (L.h0 * L.h0) / o.N2(o.D, n, g) * Lmom2;
}

// LU_solve (mod_nodal.f90:829-897): no pivoting; the near-zero test reads the
// input matrix diagonal against the single-precision literal 10e-5.
static void lu_solve(Ora& o, int nt, int msize, const std::vector<double>& mat, const std::vector<double>& b,
                     std::vector<double>& x) {
  auto MI = [&](int i, int j) { return (size_t)(i - 1) + (size_t)msize * (j - 1); };
  std::vector<double> U(mat.begin(), mat.begin() + (size_t)msize * msize), L((size_t)msize * msize, 0.0), y(msize);
  for (int i = 1; i <= msize; ++i) {
    if (std::fabs(mat[MI(i, i)]) < F_1em4) {
      char buf[160];
      std::snprintf(buf, sizeof buf, "error in matrix decomp: diagonal elements close to zero at I = %d, J = %d, K = %d",
                    o.ix[nt - 1], o.iy[nt - 1], o.iz[nt - 1]);
      throw OraError(ORA_ERR_PIVOT, buf);
    }
    L[MI(i, i)] = 1.0;
    for (int j = i + 1; j <= msize; ++j) {
      double piv = U[MI(j, i)] / U[MI(i, i)];
      L[MI(j, i)] = piv;
      for (int k = i; k <= msize; ++k) U[MI(j, k)] = U[MI(j, k)] - piv * U[MI(i, k)];
      U[MI(j, i)] = 0.0;
    }
  }
  y[0] = b[0];
  for (int i = 2; i <= msize; ++i) {
    double isum = 0.0;
    for (int k = 1; k <= i - 1; ++k) isum = isum + L[MI(i, k)] * y[k - 1];
    y[i - 1] = b[i - 1] - isum;
  }
  x.assign(msize, 0.0);
  x[msize - 1] = y[msize - 1] / U[MI(msize, msize)];
  for (int i = msize - 1; i >= 1; --i) {
    double isum = 0.0;
    for (int k = i + 1; k <= msize; ++k) isum = isum + U[MI(i, k)] * x[k - 1];
    x[i - 1] = (y[i - 1] - isum) / U[MI(i, i)];
  }
}

// get_a2matvec (mod_nodal.f90:769-825); in the transient mode (cmode 2)
// the source already holds -exsrc
static void get_a2matvec(Ora& o, int u, int n, std::vector<double>& A, std::vector<double>& b) {
  int G = o.ng;
  std::vector<double> Bf(G, 0.0);
  double h = hdir(o, u, n);
  std::vector<double>& S = (u == 1) ? o.S1 : (u == 2) ? o.S2 : o.S3;
  for (int g = 1; g <= G; ++g) {
    double Sv = (o.cmode == 2) ? 0.25 * (h * h) / o.N2(o.D, n, g) * o.N2(S, n, g)
                               : 0.25 * (h * h) / o.N2(o.D, n, g) * (o.N2(S, n, g) - o.N2(o.exsrc, n, g));
    for (int hh = 1; hh <= G; ++hh) {
      if (hh == g) A[(g - 1) + G * (hh - 1)] = o.Bm(o.Bcp, g, hh) * o.Ep[g - 1] + 3.0;
      else A[(g - 1) + G * (hh - 1)] = o.Bm(o.Bcp, g, hh) * o.Ep[g - 1];
      Bf[g - 1] = Bf[g - 1] + o.Bm(o.Bcp, g, hh) * o.N2(o.f0, n, hh);
    }
    o.Lm2[g - 1] = tlupd2(o, u, n, g);
    b[g - 1] = Bf[g - 1] - o.Ep[g - 1] * o.Lm2[g - 1] + Sv;
  }
}

// get_a4 (mod_nodal.f90:740-765)
static void get_a4(Ora& o, const std::vector<double>& a2, std::vector<double>& a4) {
  for (int g = 1; g <= o.ng; ++g) {
    double Bf = 0.0;
    for (int h = 1; h <= o.ng; ++h) Bf = Bf + o.Bm(o.Bcp, g, h) * a2[h - 1];
    a4[g - 1] = o.Bp[g - 1] * (Bf + o.Lm2[g - 1]);
  }
}

// get_a3 (mod_nodal.f90:702-736)
static void get_a3(Ora& o, int cp, const std::vector<double>& a1, const std::vector<double>& Lmn1, std::vector<double>& a3) {
  std::vector<double>& Bc = (cp == 1) ? o.Bcn : o.Bcp;
  std::vector<double>& Ac = (cp == 1) ? o.An : o.Ap;
  for (int g = 1; g <= o.ng; ++g) {
    double Bf = 0.0;
    for (int h = 1; h <= o.ng; ++h) Bf = Bf + o.Bm(Bc, g, h) * a1[h - 1];
    a3[g - 1] = Ac[g - 1] * (Bf + Lmn1[g - 1]);
  }
}

// get_a1matvec_first (mod_nodal.f90:483-552)
static void get_a1matvec_first(Ora& o, int bc, int u, int p, std::vector<double>& A, std::vector<double>& b) {
  int G = o.ng;
  double dn = hdir(o, u, p);
  int sf = 2 * u;
  auto AM = [&](int g, int h) -> double& { return A[(g - 1) + G * (h - 1)]; };
  for (int g = 1; g <= G; ++g) {
    o.Lp1[g - 1] = tlupd1(o, u, p, g);
    double Pp = 2.0 * o.N2(o.D, p, g) / dn;
    double dcv = o.X3(o.dc, p, g, sf);
    double Apg = o.Ap[g - 1], Fpg = o.Fp[g - 1], Gpg = o.Gp[g - 1], Hpg = o.Hp[g - 1];
    double a2 = o.a2p[g - 1], a4 = o.a4p[g - 1], L1 = o.Lp1[g - 1], f = o.N2(o.f0, p, g);
    if (bc == 2) {
      for (int h = 1; h <= G; ++h) {
        double Bc = o.Bm(o.Bcp, g, h);
        if (h == g) AM(g, g) = Pp * (Bc * Fpg + 1.0);
        else AM(g, h) = Pp * Bc * Fpg;
      }
      b[g - 1] = Pp * (3.0 * a2 + Gpg * a4 - Fpg * L1);
    } else if (bc == 1) {
      for (int h = 1; h <= G; ++h) {
        double Bc = o.Bm(o.Bcp, g, h);
        if (h == g) AM(g, g) = -dcv * (1.0 + Apg * Bc) - 2.0 * Pp * (Apg * Bc * Hpg + 1.0);
        else AM(g, h) = -dcv * Apg * Bc - 2.0 * Pp * Apg * Bc * Hpg;
      }
      b[g - 1] = 2.0 * Pp * (Apg * Hpg * L1 - 3.0 * a2 - Gpg * a4) - dcv * (a2 + a4 + f - Apg * L1);
    } else {
      for (int h = 1; h <= G; ++h) {
        double Bc = o.Bm(o.Bcp, g, h);
        if (h == g) AM(g, g) = dcv * (1.0 + Apg * Bc);
        else AM(g, h) = dcv * Apg * Bc;
      }
      b[g - 1] = dcv * (a2 + a4 + f - Apg * L1);
    }
  }
}

// get_a1matvec_last (mod_nodal.f90:556-626)
static void get_a1matvec_last(Ora& o, int bc, int u, int n, std::vector<double>& A, std::vector<double>& b) {
  int G = o.ng;
  double dn = hdir(o, u, n);
  int sf = 2 * u - 1;
  auto AM = [&](int g, int h) -> double& { return A[(g - 1) + G * (h - 1)]; };
  for (int g = 1; g <= G; ++g) {
    o.Ln1[g - 1] = o.Lp1[g - 1];
    double Pn = 2.0 * o.N2(o.D, n, g) / dn;
    double dcv = o.X3(o.dc, n, g, sf);
    double Ang = o.An[g - 1], Fng = o.Fn[g - 1], Gng = o.Gn[g - 1], Hng = o.Hn[g - 1];
    double a2 = o.a2n[g - 1], a4 = o.a4n[g - 1], L1 = o.Ln1[g - 1], f = o.N2(o.f0, n, g);
    if (bc == 2) {
      for (int h = 1; h <= G; ++h) {
        double Bc = o.Bm(o.Bcn, g, h);
        if (h == g) AM(g, g) = -Pn * (Bc * Fng + 1.0);
        else AM(g, h) = -Pn * Bc * Fng;
      }
      b[g - 1] = Pn * (3.0 * a2 + Gng * a4 + Fng * L1);
    } else if (bc == 1) {
      for (int h = 1; h <= G; ++h) {
        double Bc = o.Bm(o.Bcn, g, h);
        if (h == g) AM(g, g) = dcv * (1.0 + Ang * Bc) + 2.0 * Pn * (Ang * Bc * Hng + 1.0);
        else AM(g, h) = dcv * Ang * Bc + 2.0 * Pn * Ang * Bc * Hng;
      }
      b[g - 1] = -2.0 * Pn * (Ang * Hng * L1 + 3.0 * a2 + Gng * a4) - dcv * (a2 + a4 + f + Ang * L1);
    } else {
      for (int h = 1; h <= G; ++h) {
        double Bc = o.Bm(o.Bcn, g, h);
        if (h == g) AM(g, g) = dcv * (1.0 + Ang * Bc);
        else AM(g, h) = dcv * Ang * Bc;
      }
      b[g - 1] = -dcv * (a2 + a4 + f + Ang * L1);
    }
  }
}

// get_a1matvec (mod_nodal.f90:630-698), including the ADF pairing at :693-694
static void get_a1matvec(Ora& o, int u, int n, int p, std::vector<double>& A, std::vector<double>& b) {
  int G = o.ng, G2 = 2 * o.ng;
  double hn = hdir(o, u, n), hp = hdir(o, u, p);
  int sf = 2 * u - 1;
  auto AM = [&](int g, int h) -> double& { return A[(g - 1) + G2 * (h - 1)]; };
  std::vector<double> Pn(G), Pp(G);
  for (int g = 1; g <= G; ++g) {
    o.Ln1[g - 1] = o.Lp1[g - 1];
    o.Lp1[g - 1] = tlupd1(o, u, p, g);
    Pn[g - 1] = 2.0 * o.N2(o.D, n, g) / hn;
    Pp[g - 1] = 2.0 * o.N2(o.D, p, g) / hp;
    for (int h = 1; h <= G; ++h) {
      if (h == g) {
        AM(g, g) = -Pn[g - 1] * (o.Bm(o.Bcn, g, h) * o.Fn[g - 1] + 1.0);
        AM(g, g + G) = Pp[g - 1] * (o.Bm(o.Bcp, g, h) * o.Fp[g - 1] + 1.0);
      } else {
        AM(g, h) = -Pn[g - 1] * o.Bm(o.Bcn, g, h) * o.Fn[g - 1];
        AM(g, h + G) = Pp[g - 1] * o.Bm(o.Bcp, g, h) * o.Fp[g - 1];
      }
    }
    b[g - 1] = Pn[g - 1] * (3.0 * o.a2n[g - 1] + o.Gn[g - 1] * o.a4n[g - 1] + o.Fn[g - 1] * o.Ln1[g - 1]) +
               Pp[g - 1] * (3.0 * o.a2p[g - 1] + o.Gp[g - 1] * o.a4p[g - 1] - o.Fp[g - 1] * o.Lp1[g - 1]);
  }
  for (int g = 1; g <= G; ++g) {
    double dcn = o.X3(o.dc, n, g, sf), dcp = o.X3(o.dc, p, g, sf + 1);
    for (int h = 1; h <= G; ++h) {
      if (h == g) {
        AM(g + G, g) = dcn * (o.Bm(o.Bcn, g, h) * o.An[g - 1] + 1.0);
        AM(g + G, g + G) = dcp * (o.Bm(o.Bcp, g, h) * o.Ap[g - 1] + 1.0);
      } else {
        AM(g + G, h) = dcn * o.Bm(o.Bcn, g, h) * o.An[g - 1];
        AM(g + G, h + G) = dcp * o.Bm(o.Bcp, g, h) * o.Ap[g - 1];
      }
    }
    b[g + G - 1] = dcp * (o.a2p[g - 1] + o.a4p[g - 1] + o.N2(o.f0, p, g) - o.An[g - 1] * o.Ln1[g - 1]) -
                   dcn * (o.a2n[g - 1] + o.a4n[g - 1] + o.N2(o.f0, n, g) + o.Ap[g - 1] * o.Lp1[g - 1]);
  }
}

// get_coefs_first (mod_nodal.f90:375-406)
static void get_coefs_first(Ora& o, int bc, int u, int p) {
  int G = o.ng;
  std::vector<double> A((size_t)G * G), b(G);
  get_a2matvec(o, u, p, A, b);
  lu_solve(o, p, G, A, b, o.a2p);
  get_a4(o, o.a2p, o.a4p);
  get_a1matvec_first(o, bc, u, p, A, b);
  lu_solve(o, p, G, A, b, o.a1p);
  get_a3(o, 2, o.a1p, o.Lp1, o.a3p);
}

// get_coefs_last (mod_nodal.f90:410-438)
static void get_coefs_last(Ora& o, int bc, int u, int n) {
  int G = o.ng;
  std::vector<double> A((size_t)G * G), b(G);
  o.a2n = o.a2p;
  o.a4n = o.a4p;
  get_a1matvec_last(o, bc, u, n, A, b);
  lu_solve(o, n, G, A, b, o.a1n);
  get_a3(o, 1, o.a1n, o.Ln1, o.a3n);
}

// get_coefs (mod_nodal.f90:442-479)
static void get_coefs(Ora& o, int u, int n, int p) {
  int G = o.ng;
  std::vector<double> A((size_t)G * G), b(G), R((size_t)4 * G * G), s(2 * G), sol;
  o.a2n = o.a2p;
  o.a4n = o.a4p;
  get_a2matvec(o, u, p, A, b);
  lu_solve(o, p, G, A, b, o.a2p);
  get_a4(o, o.a2p, o.a4p);
  get_a1matvec(o, u, n, p, R, s);
  lu_solve(o, n, 2 * G, R, s, sol);
  for (int g = 0; g < G; ++g) o.a1n[g] = sol[g];
  get_a3(o, 1, o.a1n, o.Ln1, o.a3n);
}

// nodal_coup_upd (mod_nodal.f90:282-371); which = 0 both, 1 p only, 2 n only
static void nodal_coup_upd(Ora& o, int u, const std::vector<double>& a1, const std::vector<double>& a2,
                           const std::vector<double>& a3, const std::vector<double>& a4, int n, int p, int which) {
  int sf = 2 * u - 1;
  double dh = (which == 1) ? hdir(o, u, p) : hdir(o, u, n);
  for (int g = 1; g <= o.ng; ++g) {
    if (which == 0) {
      double jp = -2.0 * o.N2(o.D, n, g) / dh * (a1[g - 1] + 3.0 * a2[g - 1] + o.Hn[g - 1] * a3[g - 1] + o.Gn[g - 1] * a4[g - 1]);
      double ndpr = o.X3(o.dn, n, g, sf);
      double fn = o.N2(o.f0, n, g), fp = o.N2(o.f0, p, g);
      o.X3(o.dn, n, g, sf) = (o.X3(o.df, n, g, sf) * (fn - fp) - jp) / (fn + fp);
      o.X3(o.dn, p, g, sf + 1) = o.X3(o.dn, n, g, sf);
      double nder = std::fabs(o.X3(o.dn, n, g, sf) - ndpr);
      if (nder > o.ndmax) { o.ndmax = nder; o.im = o.ix[n - 1]; o.jm = o.iy[n - 1]; o.km = o.iz[n - 1]; }
    } else if (which == 1) {
      double jp = -2.0 * o.N2(o.D, p, g) / dh * (a1[g - 1] - 3.0 * a2[g - 1] + o.Hp[g - 1] * a3[g - 1] - o.Gp[g - 1] * a4[g - 1]);
      double ndpr = o.X3(o.dn, p, g, sf + 1);
      o.X3(o.dn, p, g, sf + 1) = -(jp / o.N2(o.f0, p, g) + o.X3(o.df, p, g, sf + 1));
      double nder = std::fabs(o.X3(o.dn, p, g, sf + 1) - ndpr);
      if (nder > o.ndmax) { o.ndmax = nder; o.im = o.ix[p - 1]; o.jm = o.iy[p - 1]; o.km = o.iz[p - 1]; }
    } else {
      double jp = -2.0 * o.N2(o.D, n, g) / dh * (a1[g - 1] + 3.0 * a2[g - 1] + o.Hn[g - 1] * a3[g - 1] + o.Gn[g - 1] * a4[g - 1]);
      double ndpr = o.X3(o.dn, n, g, sf);
      o.X3(o.dn, n, g, sf) = -(jp / o.N2(o.f0, n, g) - o.X3(o.df, n, g, sf));
      double nder = std::fabs(o.X3(o.dn, n, g, sf) - ndpr);
      if (nder > o.ndmax) { o.ndmax = nder; o.im = o.ix[n - 1]; o.jm = o.iy[n - 1]; o.km = o.iz[n - 1]; }
    }
  }
}

static void shift_p_to_n(Ora& o) {
  o.Bcn = o.Bcp;
  o.An = o.Ap; o.Bn = o.Bp; o.En = o.Ep; o.Fn = o.Fp; o.Gn = o.Gp; o.Hn = o.Hp;
}

// nodal_update (mod_nodal.f90:18-147, SANM) and nodal_update_pnm
// (mod_nodal.f90:151-278, PNM constants at :180-182)
static void nodal_update(Ora& o, int cal_mode, bool pnm) {
  int G = o.ng;
  o.a1n.assign(G, 0); o.a2n = o.a3n = o.a4n = o.a1p = o.a2p = o.a3p = o.a4p = o.a1n;
  o.Ln1.assign(G, 0); o.Lp1.assign(G, 0);
  o.Bcn.assign((size_t)G * G, 0); o.Bcp = o.Bcn;
  o.An.assign(G, 0); o.Bn = o.En = o.Fn = o.Gn = o.Hn = o.An;
  o.Ap = o.Bp = o.Ep = o.Fp = o.Gp = o.Hp = o.An;
  o.Lm2.assign(G, 0);
  if (pnm) {
    for (int g = 0; g < G; ++g) {
      o.An[g] = 1.0 / 15.0; o.Bn[g] = 1.0 / 35.0; o.En[g] = 2.0 / 7.0;
      o.Fn[g] = 2.0 / 5.0; o.Gn[g] = 10.0; o.Hn[g] = 6.0;
    }
    o.Ap = o.An; o.Bp = o.Bn; o.Ep = o.En; o.Fp = o.Fn; o.Gp = o.Gn; o.Hp = o.Hn;
  }
  o.cmode = cal_mode;
  get_source(o);
  auto abefgh = [&](int p, int u) { if (!pnm) get_ABEFGH(o, p, u, o.Ap, o.Bp, o.Ep, o.Fp, o.Gp, o.Hp); };
  // x sweep
  for (int k = 1; k <= o.nzz; ++k)
    for (int j = 1; j <= o.nyy; ++j) {
      int p = o.XYZ(o.ysmin[j - 1], j, k);
      get_B(o, 1, p, o.Bcp);
      abefgh(p, 1);
      get_coefs_first(o, o.xwest, 1, p);
      nodal_coup_upd(o, 1, o.a1p, o.a2p, o.a3p, o.a4p, 0, p, 1);
      for (int i = o.ysmin[j - 1]; i <= o.ysmax[j - 1] - 1; ++i) {
        int n = o.XYZ(i, j, k);
        p = o.XYZ(i + 1, j, k);
        shift_p_to_n(o);
        get_B(o, 1, p, o.Bcp);
        abefgh(p, 1);
        get_coefs(o, 1, n, p);
        nodal_coup_upd(o, 1, o.a1n, o.a2n, o.a3n, o.a4n, n, p, 0);
      }
      int n = o.XYZ(o.ysmax[j - 1], j, k);
      shift_p_to_n(o);
      get_coefs_last(o, o.xeast, 1, n);
      nodal_coup_upd(o, 1, o.a1n, o.a2n, o.a3n, o.a4n, n, 0, 2);
    }
  // y sweep
  for (int k = 1; k <= o.nzz; ++k)
    for (int i = 1; i <= o.nxx; ++i) {
      int p = o.XYZ(i, o.xsmin[i - 1], k);
      get_B(o, 2, p, o.Bcp);
      abefgh(p, 2);
      get_coefs_first(o, o.ysouth, 2, p);
      nodal_coup_upd(o, 2, o.a1p, o.a2p, o.a3p, o.a4p, 0, p, 1);
      for (int j = o.xsmin[i - 1]; j <= o.xsmax[i - 1] - 1; ++j) {
        int n = o.XYZ(i, j, k);
        p = o.XYZ(i, j + 1, k);
        shift_p_to_n(o);
        get_B(o, 2, p, o.Bcp);
        abefgh(p, 2);
        get_coefs(o, 2, n, p);
        nodal_coup_upd(o, 2, o.a1n, o.a2n, o.a3n, o.a4n, n, p, 0);
      }
      int n = o.XYZ(i, o.xsmax[i - 1], k);
      shift_p_to_n(o);
      get_coefs_last(o, o.ynorth, 2, n);
      nodal_coup_upd(o, 2, o.a1n, o.a2n, o.a3n, o.a4n, n, 0, 2);
    }
  // z sweep
  for (int j = 1; j <= o.nyy; ++j)
    for (int i = o.ysmin[j - 1]; i <= o.ysmax[j - 1]; ++i) {
      int p = o.XYZ(i, j, 1);
      get_B(o, 3, p, o.Bcp);
      abefgh(p, 3);
      get_coefs_first(o, o.zbott, 3, p);
      nodal_coup_upd(o, 3, o.a1p, o.a2p, o.a3p, o.a4p, 0, p, 1);
      for (int k = 1; k <= o.nzz - 1; ++k) {
        int n = o.XYZ(i, j, k);
        p = o.XYZ(i, j, k + 1);
        shift_p_to_n(o);
        get_B(o, 3, p, o.Bcp);
        abefgh(p, 3);
        get_coefs(o, 3, n, p);
        nodal_coup_upd(o, 3, o.a1n, o.a2n, o.a3n, o.a4n, n, p, 0);
      }
      int n = o.XYZ(i, j, o.nzz);
      shift_p_to_n(o);
      get_coefs_last(o, o.ztop, 3, n);
      nodal_coup_upd(o, 3, o.a1n, o.a2n, o.a3n, o.a4n, n, 0, 2);
    }
  if (o.ndmax > 1.e3) {
    char buf[160];
    std::snprintf(buf, sizeof buf, "max. change in nodal coupling coefficient = %.1f: the two-node nonlinear iteration seems not stable", o.ndmax);
    throw OraError(ORA_ERR_DIVERGED, buf);
  }
}

// nodal_upd (mod_cmfd.f90:339-383)
static void nodal_upd(Ora& o, int nmode) {
  o.ndmax = 0.0;
  nodal_update(o, nmode, o.kern != "SANM");
  matrix_setup(o, 0);
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// outer (mod_cmfd.f90:415-509) and outer_ad (mod_cmfd.f90:602-699)
static void outer(Ora& o, bool adj, int popt, int max_outers) {
  double st = now_s();
  int N = o.nnod, G = o.ng;
  matrix_setup(o, 1);
  bool& first = adj ? o.outer_ad_first : o.outer_first;
  if (first && (adj ? popt > 0 : true)) {
    o.f0.assign((size_t)N * G, 1.0);
    o.fs0.assign(N, 0.0);
    o.s0.assign((size_t)N * G, 0.0);
    o.Ke = 1.0;
    fsrc(o, o.fs0, adj);
    first = false;
  }
  if (o.s0.empty()) o.s0.assign((size_t)N * G, 0.0);
  std::vector<double> fs0c(N), bs(N), f0c((size_t)N * G), errn(N, 1.0), erro(N);
  double f = integrate(o, o.fs0), fc, Keo, e1, e2;
  e1 = integrate(o, errn);
  o.trace.clear();
  o.t_cmfd += now_s() - st;
  int p;
  int cap = (max_outers > 0) ? std::min(max_outers, o.nout) : o.nout;
  for (p = 1; p <= cap; ++p) {
    st = now_s();
    TraceRec tr{};
    tr.p = p;
    fc = f; fs0c = o.fs0; f0c = o.f0; Keo = o.Ke; erro = errn;
    if (!adj) {
      for (int g = 1; g <= G; ++g) {
        tsrc(o, g, o.Ke, bs, false);
        bicg(o, o.nin, g, bs, &o.f0[(size_t)N * (g - 1)]);
      }
    } else {
      for (int g = G; g >= 1; --g) {
        tsrc(o, g, o.Ke, bs, true);
        bicg(o, o.nin, g, bs, &o.f0[(size_t)N * (g - 1)]);
      }
    }
    fsrc(o, o.fs0, adj);
    for (int n = 0; n < N; ++n) errn[n] = o.fs0[n] - fs0c[n];
    e2 = l2norm(errn);
    if (p % o.nac == 0) { fiss_extrp(e1, e2, errn, o.fs0); tr.extrapolated = 1; }
    e1 = e2;
    f = integrate(o, o.fs0);
    o.Ke = Keo * f / fc;
    double ser = rele(o, o.fs0, fs0c);
    double fer = releg(o, o.f0, f0c);
    o.t_cmfd += now_s() - st;
    if (p % o.nupd == 0 && o.kern != " FDM" && (!adj || popt > 0)) {
      st = now_s();
      nodal_upd(o, adj ? 0 : 1);
      o.t_nodal += now_s() - st;
      tr.nodal = 1; tr.ndmax = o.ndmax; tr.im = o.im; tr.jm = o.jm; tr.km = o.km;
    }
    tr.k = o.Ke; tr.ser = ser; tr.fer = fer;
    o.trace.push_back(tr);
    o.last_ser = ser; o.last_fer = fer;
    if (ser < o.serc && fer < o.ferc && o.ndmax < F_1em2) break;
  }
  o.last_outers = std::min(p, cap);
  if (max_outers > 0 && p > cap && cap < o.nout) return;   // bounded sample run
  if (p - 1 == o.nout) throw OraError(ORA_ERR_MAXOUTER, "maximum number of outer iteration is reached");
}

// PowDis (mod_cmfd.f90:1290-1333)
static void powdis(Ora& o, double* pw) {
  int N = o.nnod;
  for (int n = 0; n < N; ++n) pw[n] = 0.0;
  for (int g = 1; g <= o.ng; ++g)
    for (int n = 1; n <= N; ++n) {
      double pow = o.N2(o.f0, n, g) * o.N2(o.sigf, n, g) * o.vdel[n - 1];
      if (pow < 0.) pow = 0.;
      pw[n - 1] = pw[n - 1] + pow;
    }
  double tpow = 0.0;
  for (int n = 0; n < N; ++n) tpow = tpow + pw[n];
  if (tpow <= 0) throw OraError(ORA_ERR_ZEROPOWER, "total nodes power is zero or less");
  for (int n = 0; n < N; ++n) pw[n] = pw[n] / tpow;
}

// Output edits of control::forward (mod_control.f90:33-44), numeric part.
// fx(i,j,k) is the node field on the box, 0 where there is no node.
static std::vector<double> box_field(const Ora& o, const double* fn) {
  std::vector<double> fx((size_t)o.nxx * o.nyy * o.nzz, 0.0);
  for (int n = 0; n < o.nnod; ++n)
    fx[(o.ix[n] - 1) + (size_t)o.nxx * ((o.iy[n] - 1) + (size_t)o.nyy * (o.iz[n] - 1))] = fn[n];
  return fx;
}

// AsmPow (mod_io.f90:3267-3403): axially averaged node values, area-weighted
// assembly averages, normalised so that the non-zero assemblies average 1,
// and the first maximum in (j, i) order.  fasm is (nx,ny); imax/jmax 1-based.
static void asmpow(Ora& o, const double* fn, double* fasm, int* imax, int* jmax) {
  const std::vector<double> fx = box_field(o, fn);
  auto FX = [&](int i, int j, int k) { return fx[(i - 1) + (size_t)o.nxx * ((j - 1) + (size_t)o.nyy * (k - 1))]; };
  std::vector<double> fnode((size_t)o.nxx * o.nyy, 0.0);
  for (int j = 1; j <= o.nyy; ++j)
    for (int i = o.ysmin[j - 1]; i <= o.ysmax[j - 1]; ++i) {
      double summ = 0.0, vsumm = 0.0;
      for (int k = 1; k <= o.nzz; ++k) {
        summ = summ + FX(i, j, k) * o.zdel[k - 1];
        vsumm = vsumm + o.zdel[k - 1];
      }
      fnode[(i - 1) + (size_t)o.nxx * (j - 1)] = summ / vsumm;
    }
  int nfuel = 0;
  double totp = 0.0;
  int ys = 1, yf = 0;
  for (int j = 1; j <= o.ny; ++j) {
    yf += o.ydiv[j - 1];
    int xf = 0, xs = 1;
    for (int i = 1; i <= o.nx; ++i) {
      xf += o.xdiv[i - 1];
      double summ = 0.0, vsumm = 0.0;
      for (int ly = ys; ly <= yf; ++ly)
        for (int lx = xs; lx <= xf; ++lx) {
          summ = summ + fnode[(lx - 1) + (size_t)o.nxx * (ly - 1)] * o.xdel[lx - 1] * o.ydel[ly - 1];
          vsumm = vsumm + o.xdel[lx - 1] * o.ydel[ly - 1];
        }
      double& fa = fasm[(i - 1) + (size_t)o.nx * (j - 1)];
      fa = summ / vsumm;
      xs += o.xdiv[i - 1];
      if (fa > 0.0) { ++nfuel; totp = totp + fa; }
    }
    ys += o.ydiv[j - 1];
  }
  *imax = 1;
  *jmax = 1;
  double fmax = 0.0;
  for (int j = 1; j <= o.ny; ++j)
    for (int i = 1; i <= o.nx; ++i) {
      double& fa = fasm[(i - 1) + (size_t)o.nx * (j - 1)];
      if (totp > 0.) fa = (double)(float)nfuel / totp * fa;   // REAL(nfuel) is default (single) real
      if (fa > fmax) { *imax = i; *jmax = j; fmax = fa; }
    }
}

// AxiPow (mod_io.f90:3406-3498): node values summed over each axial region
// (zdiv planes) divided by its volume, normalised so the non-zero regions
// average 1; the first maximum.  faxi is (nz); kmax 1-based.
static void axipow(Ora& o, const double* fn, double* faxi, int* kmax) {
  const std::vector<double> fx = box_field(o, fn);
  int nfuel = 0, ztot = 0;
  double totp = 0.0;
  for (int k = 1; k <= o.nz; ++k) {
    double summ = 0.0, vsumm = 0.0;
    for (int lz = 1; lz <= o.zdiv[k - 1]; ++lz) {
      ++ztot;
      for (int j = 1; j <= o.nyy; ++j)
        for (int i = o.ysmin[j - 1]; i <= o.ysmax[j - 1]; ++i) {
          summ = summ + fx[(i - 1) + (size_t)o.nxx * ((j - 1) + (size_t)o.nyy * (ztot - 1))];
          vsumm = vsumm + o.vdel[o.XYZ(i, j, ztot) - 1];
        }
    }
    faxi[k - 1] = summ / vsumm;
    if (faxi[k - 1] > 0.0) { ++nfuel; totp = totp + faxi[k - 1]; }
  }
  double fmax = 0.0;
  *kmax = 1;
  for (int k = 1; k <= o.nz; ++k) {
    faxi[k - 1] = (double)(float)nfuel / totp * faxi[k - 1];
    if (faxi[k - 1] > fmax) { *kmax = k; fmax = faxi[k - 1]; }
  }
}

// AsmFlux (mod_io.f90:3501-3644): per group, volume-weighted axial average
// of the node flux, area-weighted assembly averages, scaled by
// norm / sum(positive assemblies) * norm when norm is given (forward calls
// it with 1.0); negf = 1 when an assembly average is negative.
static void asmflux(Ora& o, const double* f, bool has_norm, double norm, double* fasm, int* negf) {
  const int G = o.ng;
  std::vector<double> fnode((size_t)o.nxx * o.nyy * G, 0.0);
  for (int g = 1; g <= G; ++g) {
    const std::vector<double> fx = box_field(o, f + (size_t)o.nnod * (g - 1));
    for (int j = 1; j <= o.nyy; ++j)
      for (int i = o.ysmin[j - 1]; i <= o.ysmax[j - 1]; ++i) {
        double summ = 0.0, vsumm = 0.0;
        for (int k = 1; k <= o.nzz; ++k) {
          const double v = fx[(i - 1) + (size_t)o.nxx * ((j - 1) + (size_t)o.nyy * (k - 1))];
          summ = summ + v * o.xdel[i - 1] * o.ydel[j - 1] * o.zdel[k - 1];
          vsumm = vsumm + o.xdel[i - 1] * o.ydel[j - 1] * o.zdel[k - 1];
        }
        fnode[(i - 1) + (size_t)o.nxx * ((j - 1) + (size_t)o.nyy * (g - 1))] = summ / vsumm;
      }
  }
  *negf = 0;
  std::vector<double> totp(G, 0.0);
  for (int g = 1; g <= G; ++g) {
    int ys = 1, yf = 0;
    for (int j = 1; j <= o.ny; ++j) {
      yf += o.ydiv[j - 1];
      int xf = 0, xs = 1;
      for (int i = 1; i <= o.nx; ++i) {
        xf += o.xdiv[i - 1];
        double summ = 0.0, vsumm = 0.0;
        for (int ly = ys; ly <= yf; ++ly)
          for (int lx = xs; lx <= xf; ++lx) {
            summ = summ + fnode[(lx - 1) + (size_t)o.nxx * ((ly - 1) + (size_t)o.nyy * (g - 1))] * o.xdel[lx - 1] *
                              o.ydel[ly - 1];
            vsumm = vsumm + o.xdel[lx - 1] * o.ydel[ly - 1];
          }
        double& fa = fasm[(i - 1) + (size_t)o.nx * ((j - 1) + (size_t)o.ny * (g - 1))];
        fa = summ / vsumm;
        xs += o.xdiv[i - 1];
        if (fa > 0.0) totp[g - 1] = totp[g - 1] + fa;
        if (fa < 0.0) *negf = 1;
      }
      ys += o.ydiv[j - 1];
    }
  }
  if (has_norm)
    for (int g = 1; g <= G; ++g)
      for (int q = 0; q < o.nx * o.ny; ++q) {
        double& fa = fasm[q + (size_t)o.nx * o.ny * (g - 1)];
        fa = norm / totp[g - 1] * fa * norm;
      }
}

// reactivity (mod_trans.f90:648-688): adjoint-weighted balance of the
// current state, rho = (src - lea - rem) / fde, with the scattering-in and
// fission sources, the net leakage of Lxyz and the removal sigrp.
static double reactivity(Ora& o, const double* af, const double* sigrp) {
  const int N = o.nnod, G = o.ng;
  double src = 0., rem = 0., lea = 0., fde = 0.;
  std::vector<double> scg(N);
  for (int g = 1; g <= G; ++g) {
    std::fill(scg.begin(), scg.end(), 0.0);
    for (int h = 1; h <= G; ++h)
      for (int n = 1; n <= N; ++n)
        if (g != h) scg[n - 1] = scg[n - 1] + o.SG(o.sigs, n, h, g) * o.N2(o.f0, n, h);
    for (int n = 1; n <= N; ++n) {
      double L1, L2, L3;
      lxyz(o, n, g, L1, L2, L3);
      const double L = L1 + L2 + L3;
      if (!o.Lt.empty()) o.N2(o.Lt, n, g) = L;   // L(n,g) of the transient source
      const double a = af[(n - 1) + (size_t)N * (g - 1)];
      const double chi = o.M2(o.chi, o.mat[n - 1], g);
      src = src + a * (scg[n - 1] + chi * o.fs0[n - 1]) * o.vdel[n - 1];
      rem = rem + a * sigrp[(n - 1) + (size_t)N * (g - 1)] * o.N2(o.f0, n, g) * o.vdel[n - 1];
      lea = lea + a * L * o.vdel[n - 1];
      fde = fde + a * chi * o.fs0[n - 1] * o.vdel[n - 1];
    }
  }
  return (src - lea - rem) / fde;
}

// calc_beta (mod_trans.f90:692-746): core-averaged delayed neutron fraction
// weighted by af, from the delayed fractions ibeta(nmat, nf).
static double calc_beta(Ora& o, const double* af, int nf, const double* ibeta) {
  const int N = o.nnod, G = o.ng;
  std::vector<double> vdum(N, 0.0), vdum2(N, 0.0);
  for (int g = 1; g <= G; ++g)
    for (int n = 1; n <= N; ++n) vdum[n - 1] = vdum[n - 1] + o.N2(o.nuf, n, g) * o.N2(o.f0, n, g);
  for (int g = 1; g <= G; ++g)
    for (int n = 1; n <= N; ++n)
      vdum2[n - 1] = vdum2[n - 1] + o.M2(o.chi, o.mat[n - 1], g) * vdum[n - 1] * af[(n - 1) + (size_t)N * (g - 1)];
  const double F = integrate(o, vdum2);
  double beta = 0.0;
  for (int i = 1; i <= nf; ++i) {
    std::fill(vdum2.begin(), vdum2.end(), 0.0);
    for (int g = 1; g <= G; ++g)
      for (int n = 1; n <= N; ++n)
        vdum2[n - 1] = vdum2[n - 1] + o.M2(o.chi, o.mat[n - 1], g) * ibeta[(o.mat[n - 1] - 1) + (size_t)o.nmat * (i - 1)] *
                                          vdum[n - 1] * af[(n - 1) + (size_t)N * (g - 1)];
    beta = beta + integrate(o, vdum2) / F;
  }
  return beta;
}

// ===========================================================================
// Rod ejection transient (mod_trans.f90:17-160, 332-640; mod_cmfd.f90:800-952,
// 1068-1095), without thermal-hydraulics and %XTAB
// ===========================================================================

// TSrcTr (mod_cmfd.f90:1068-1095): zero-fills all of s0, as TSrc does
static void tsrctr(Ora& o, int g, std::vector<double>& bs) {
  std::fill(o.s0.begin(), o.s0.end(), 0.0);
  for (int h = 1; h <= o.ng; ++h)
    for (int n = 1; n <= o.nnod; ++n)
      if (g != h) o.N2(o.s0, n, g) = o.N2(o.s0, n, g) + o.SG(o.sigs, n, h, g) * o.N2(o.f0, n, h);
  for (int n = 1; n <= o.nnod; ++n) {
    const int m = o.mat[n - 1];
    bs[n - 1] = (1.0 - o.tbeta[m - 1] + o.dfis[n - 1]) * o.M2(o.chi, m, g) * o.fs0[n - 1] + o.N2(o.s0, n, g) +
                o.N2(o.exsrc, n, g);
  }
}

// get_exsrc (mod_cmfd.f90:872-952): delayed source of the step and the
// theta-method terms of the previous step
static void get_exsrc(Ora& o, double ht) {
  for (int n = 1; n <= o.nnod; ++n) {
    const int m = o.mat[n - 1];
    double dt = 0.0, dtp = 0.0;
    o.dfis[n - 1] = 0.0;
    for (int i = 0; i < Ora::nf; ++i) {
      const double pxe = std::exp(-o.lamb[i] * ht);
      double a1 = (1.0 - pxe) / (o.lamb[i] * ht);
      const double a2 = 1.0 - a1;
      a1 = a1 - pxe;
      const double c = o.c0[(n - 1) + (size_t)o.nnod * i];
      o.dfis[n - 1] = o.dfis[n - 1] + o.ibeta[i] * a2;
      dt = dt + o.lamb[i] * c * pxe + o.ibeta[i] * a1 * o.fst[n - 1];
      dtp = dtp + o.lamb[i] * c;
    }
    for (int g = 1; g <= o.ng; ++g) {
      const double chi = o.M2(o.chi, m, g);
      const double pthet = -o.N2(o.Lt, n, g) - o.N2(o.sigrp, n, g) * o.N2(o.ft, n, g) + o.N2(o.s0, n, g) +
                           (1.0 - o.tbeta[m - 1]) * chi * o.fst[n - 1] + chi * dtp;
      o.N2(o.exsrc, n, g) = chi * dt + std::exp(o.N2(o.omeg, n, g) * ht) * o.N2(o.ft, n, g) /
                                           (o.sth * o.velo[g - 1] * ht) + o.bth * pthet;
    }
  }
}

// outer_tr (mod_cmfd.f90:800-868): fixed-source outer iterations of one
// step; true when nout is reached (the reference's maxi)
static bool outer_tr(Ora& o, double ht) {
  const int N = o.nnod, G = o.ng;
  matrix_setup(o, 1);
  get_exsrc(o, ht);
  std::vector<double> fs0c(N), bs(N), f0c((size_t)N * G), errn(N, 0.0);
  double e1 = 0.0, e2;
  o.trace.clear();
  int p;
  for (p = 1; p <= o.nout; ++p) {
    TraceRec tr{};
    tr.p = p;
    fs0c = o.fs0; f0c = o.f0;
    for (int g = 1; g <= G; ++g) {
      tsrctr(o, g, bs);
      bicg(o, o.nin, g, bs, &o.f0[(size_t)N * (g - 1)]);
    }
    fsrc(o, o.fs0, false);
    for (int n = 0; n < N; ++n) errn[n] = o.fs0[n] - fs0c[n];
    e2 = l2norm(errn);
    if (p % o.nac == 0) { fiss_extrp(e1, e2, errn, o.fs0); tr.extrapolated = 1; }
    e1 = e2;
    const double ser = rele(o, o.fs0, fs0c);
    const double fer = releg(o, o.f0, f0c);
    if (p % o.nupd == 0 && o.kern != " FDM") {
      nodal_upd(o, 2);
      tr.nodal = 1; tr.ndmax = o.ndmax; tr.im = o.im; tr.jm = o.jm; tr.km = o.km;
    }
    tr.k = o.Ke; tr.ser = ser; tr.fer = fer;
    o.trace.push_back(tr);
    o.last_ser = ser; o.last_fer = fer;
    if (ser < o.serc && fer < o.ferc && o.ndmax < F_1em2) break;
  }
  o.last_outers = std::min(p, o.nout);
  return p == o.nout + 1;
}

// iPden (mod_trans.f90:561-597)
static void ipden(Ora& o) {
  o.c0.assign((size_t)o.nnod * Ora::nf, 0.0);
  for (int n = 0; n < o.nnod; ++n)
    for (int j = 0; j < Ora::nf; ++j) o.c0[n + (size_t)o.nnod * j] = o.ibeta[j] / o.lamb[j] * o.fs0[n];
}

// uPden (mod_trans.f90:601-640)
static void upden(Ora& o, double ht) {
  for (int i = 0; i < Ora::nf; ++i) {
    const double pxe = std::exp(-o.lamb[i] * ht);
    double a1 = (1.0 - pxe) / (o.lamb[i] * ht);
    const double a2 = 1.0 - a1;
    a1 = a1 - pxe;
    for (int n = 0; n < o.nnod; ++n) {
      double& c = o.c0[n + (size_t)o.nnod * i];
      c = c * pxe + o.ibeta[i] / o.lamb[i] * (a1 * o.fst[n] + a2 * o.fs0[n]);
    }
  }
}

// PowTot (mod_trans.f90:522-557)
static double powtot(Ora& o) {
  std::vector<double> pw(o.nnod, 0.0);
  for (int g = 1; g <= o.ng; ++g)
    for (int n = 1; n <= o.nnod; ++n) {
      double q = o.N2(o.f0, n, g) * o.N2(o.sigf, n, g) * o.vdel[n - 1];
      if (q < 0.) q = 0.;
      pw[n - 1] = pw[n - 1] + q;
    }
  double t = 0.0;
  for (int n = 0; n < o.nnod; ++n) t = t + pw[n];
  return t;
}

// KNE1 (mod_trans.f90:483-518): scale nu*sigf (and its rod change) by 1/k
// until k = 1.  The reference tests the loop index after the loop, so an
// exit on the tenth pass stops as well, and ten passes without an exit do
// not.
static void kne1(Ora& o) {
  int i;
  for (i = 1; i <= 10; ++i) {
    for (auto& x : o.xnuf) x = x / o.Ke;
    for (auto& x : o.fb_crod.nf) x = x / o.Ke;
    xs_updt(o);
    outer(o, false, 0, 0);
    if (std::fabs(o.Ke - 1.0) < 1.e-5) break;
  }
  if (i == 10) throw OraError(ORA_ERR_INPUT, "k-eff still not equal to one");
}

struct TransRec { double t, rho, pow; int maxi, outers; };

// trans_calc (mod_trans.f90:332-479) for thc = 0
static TransRec trans_calc(Ora& o, double ht, const std::vector<double>& af, double tpow1, double t2) {
  for (int n = 0; n < o.nb; ++n) {
    if (o.mdir[n] == 1) {
      if (t2 - o.tmove[n] > 1.e-5 && o.fbpos[n] - o.bpos[n] < 1.e-5) {
        o.bpos[n] = o.bpos[n] - ht * o.bspeed[n];
        if (o.bpos[n] < o.fbpos[n]) o.bpos[n] = o.fbpos[n];
      }
    } else if (o.mdir[n] == 2) {
      if (t2 - o.tmove[n] > 1.e-5 && o.fbpos[n] - o.bpos[n] > 1.e-5) {
        o.bpos[n] = o.bpos[n] + ht * o.bspeed[n];
        if (o.bpos[n] > o.fbpos[n]) o.bpos[n] = o.fbpos[n];
      }
    }
  }
  xs_updt(o);
  o.sigrp = o.sigr;
  for (int g = 1; g <= o.ng; ++g)
    for (int n = 1; n <= o.nnod; ++n)
      o.N2(o.sigr, n, g) = o.N2(o.sigr, n, g) + 1.0 / (o.sth * o.velo[g - 1] * ht) + o.N2(o.omeg, n, g) / o.velo[g - 1];
  o.ft = o.f0;
  o.fst = o.fs0;
  const bool maxi = outer_tr(o, ht);
  upden(o, ht);
  const double tpow2 = powtot(o);
  const double rho = reactivity(o, af.data(), o.sigrp.data());
  return TransRec{t2, rho / o.ctbeta, tpow2 / tpow1, maxi ? 1 : 0, o.last_outers};
}

// rod_eject (mod_trans.f90:17-160): the steady state (k forced to one),
// the adjoint weight, initial precursors, then the two time-step phases.
// Record 0 is t = 0 with rho in absolute units, as the reference prints it.
static std::vector<TransRec> rod_eject(Ora& o, int max_steps) {
  const int N = o.nnod, G = o.ng;
  o.omeg.assign((size_t)N * G, 0.0);
  o.Lt.assign((size_t)N * G, 0.0);
  o.dfis.assign(N, 0.0);
  xs_updt(o);
  outer(o, false, 0, 0);
  if (std::fabs(o.Ke - 1.0) > 1.e-5) kne1(o);
  outer(o, true, 0, 0);
  const std::vector<double> af = o.f0;
  outer(o, false, 0, 0);
  ipden(o);
  const double tpow1 = powtot(o);
  o.tbeta.assign(o.nmat, 0.0);
  for (int n = 0; n < o.nmat; ++n) {
    for (int j = 0; j < Ora::nf; ++j) o.tbeta[n] = o.tbeta[n] + o.ibeta[j];
    o.ctbeta = o.tbeta[0];
  }
  std::vector<TransRec> out;
  out.push_back(TransRec{0.0, reactivity(o, af.data(), o.sigr.data()), 1.0, 0, o.last_outers});
  const long imax1 = std::lround(o.tdiv / o.tstep1);
  auto more = [&]() { return max_steps < 0 || (long)out.size() <= max_steps; };
  for (long i = 1; i <= imax1 && more(); ++i) {
    const double t2 = (double)(float)i * o.tstep1;
    for (size_t q = 0; q < o.omeg.size(); ++q)
      o.omeg[q] = (i > 1 && o.bextr) ? std::log(o.f0[q] / o.ft[q]) / o.tstep1 : 0.0;
    out.push_back(trans_calc(o, o.tstep1, af, tpow1, t2));
  }
  const long imax2 = std::lround((o.ttot - o.tdiv) / o.tstep2);
  for (long i = 1; i <= imax2 && more(); ++i) {
    const double t2 = o.tdiv + (double)(float)i * o.tstep2;
    for (size_t q = 0; q < o.omeg.size(); ++q)
      o.omeg[q] = o.bextr ? std::log(o.f0[q] / o.ft[q]) / o.tstep2 : 0.0;
    out.push_back(trans_calc(o, o.tstep2, af, tpow1, t2));
  }
  return out;
}

thread_local std::string g_err;

template <class F>
static int guard(Ora* o, F&& f) {
  try {
    f();
    return ORA_OK;
  } catch (const OraError& e) {
    if (o) o->err = e.what();
    g_err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    if (o) o->err = e.what();
    g_err = e.what();
    return ORA_ERR_INPUT;
  }
}

static std::vector<double>* dvec(Ora* o, const char* name) {
  std::string s(name);
  if (s == "f0") return &o->f0;
  if (s == "fs0") return &o->fs0;
  if (s == "dn") return &o->dn;
  if (s == "df") return &o->df;
  if (s == "D") return &o->D;
  if (s == "sigr") return &o->sigr;
  if (s == "exsrc") return &o->exsrc;
  if (s == "Lt") return &o->Lt;
  if (s == "sigrp") return &o->sigrp;
  if (s == "ft") return &o->ft;
  if (s == "s0") return &o->s0;
  if (s == "c0") return &o->c0;
  if (s == "sigtr") return &o->sigtr;
  if (s == "siga") return &o->siga;
  if (s == "nuf") return &o->nuf;
  if (s == "sigf") return &o->sigf;
  if (s == "sigs") return &o->sigs;
  if (s == "chi") return &o->chi;
  if (s == "dc") return &o->dc;
  if (s == "xdel") return &o->xdel;
  if (s == "ydel") return &o->ydel;
  if (s == "zdel") return &o->zdel;
  if (s == "vdel") return &o->vdel;
  if (s == "xsigtr") return &o->xsigtr;
  if (s == "xsiga") return &o->xsiga;
  if (s == "xnuf") return &o->xnuf;
  if (s == "xsigf") return &o->xsigf;
  if (s == "xsigs") return &o->xsigs;
  if (s == "S1") return &o->S1;
  if (s == "S2") return &o->S2;
  if (s == "S3") return &o->S3;
  return nullptr;
}

static std::vector<int>* ivec(Ora* o, const char* name) {
  std::string s(name);
  if (s == "ix") return &o->ix;
  if (s == "iy") return &o->iy;
  if (s == "iz") return &o->iz;
  if (s == "mat") return &o->mat;
  if (s == "ysmin") return &o->ysmin;
  if (s == "ysmax") return &o->ysmax;
  if (s == "xsmin") return &o->xsmin;
  if (s == "xsmax") return &o->xsmax;
  if (s == "xyz") return &o->xyz;
  if (s == "ncol") return &o->ncol;
  return nullptr;
}

}  // namespace

// ===========================================================================
// C interface used by the tests through ctypes.
// ===========================================================================
extern "C" {

const char* ora_global_error() { return g_err.c_str(); }

void* ora_load_deck_text(const char* text, const char* basedir) {
  Ora* o = new Ora();
  int st = guard(o, [&] { parse_deck(*o, text, basedir ? basedir : "."); });
  if (st != ORA_OK) { delete o; return nullptr; }
  return o;
}

void* ora_load_deck(const char* path) {
  std::string text;
  int st = guard(nullptr, [&] { text = read_file(path); });
  if (st != ORA_OK) return nullptr;
  return ora_load_deck_text(text.c_str(), dirname_of(path).c_str());
}

void ora_free(void* h) { delete (Ora*)h; }
const char* ora_error(void* h) { return ((Ora*)h)->err.c_str(); }

int ora_xs_updt(void* h) { Ora* o = (Ora*)h; return guard(o, [&] { xs_updt(*o); }); }
int ora_dsigr_updt(void* h) { Ora* o = (Ora*)h; return guard(o, [&] { dsigr_updt(*o); check_xs(*o); }); }

// mode: 0 forward, 1 adjoint.  max_outers > 0 stops early after that many
// outers without the maximum-outer error (used for bounded timing samples).
// cbsearch (mod_th.f90:752-837): secant search of the boron concentration
// that makes k = 1, each step XS_updt at the iterate and a warm-started
// outer(0).  Writes at most cap iterates (bcon, k, outers of the step) and
// returns their count; the STOPs of the reference become errors.
static int cbsearch(Ora& o, double* bc_out, double* k_out, int* n_out, int cap) {
  int rec = 0;
  auto log = [&](double b, double k) {
    if (rec < cap) { bc_out[rec] = b; k_out[rec] = k; n_out[rec] = o.last_outers; }
    ++rec;
  };
  double bcon = o.fb_bcon.ref;
  xs_updt_at(o, bcon);
  outer(o, false, 0, 0);
  double bc1 = bcon, ke1 = o.Ke;
  log(bc1, ke1);
  bcon = bcon + (o.Ke - 1.) * bcon;
  xs_updt_at(o, bcon);
  outer(o, false, 0, 0);
  double bc2 = bcon, ke2 = o.Ke;
  log(bc2, ke2);
  int n = 3;
  while (true) {
    bcon = bc2 + (1.0 - ke2) / (ke1 - ke2) * (bc1 - bc2);
    xs_updt_at(o, bcon);
    outer(o, false, 0, 0);
    bc1 = bc2;
    bc2 = bcon;
    ke1 = ke2;
    ke2 = o.Ke;
    log(bcon, o.Ke);
    if (std::fabs(o.Ke - 1.0) < 1.e-5 && o.last_ser < 1.e-5 && o.last_fer < 1.e-5) break;
    ++n;
    if (bcon > 3000.) throw OraError(ORA_ERR_INPUT, "critical boron concentration exceeds the limit (3000 ppm)");
    if (bcon < 0.) throw OraError(ORA_ERR_INPUT, "critical boron concentration is not found (less than zero)");
    if (n == 20) throw OraError(ORA_ERR_MAXOUTER, "maximum iteration for critical boron search is reaching maximum");
  }
  o.bcon = bcon;
  return rec;
}

int ora_cbsearch(void* h, double* bc, double* k, int* outers, int cap, int* count) {
  Ora* o = (Ora*)h;
  return guard(o, [&] { *count = cbsearch(*o, bc, k, outers, cap); });
}

// The rod ejection transient: up to cap records (t, reactivity in dollars
// (absolute at t = 0), relative power, nout reached, outers of the step);
// max_steps >= 0 stops after that many time steps.
int ora_rodeject(void* h, double* t, double* rho, double* pw, int* maxi, int* outers, int cap, int max_steps,
                 int* count) {
  Ora* o = (Ora*)h;
  return guard(o, [&] {
    const std::vector<TransRec> r = rod_eject(*o, max_steps);
    const int n = (int)std::min((size_t)cap, r.size());
    for (int i = 0; i < n; ++i) {
      t[i] = r[i].t; rho[i] = r[i].rho; pw[i] = r[i].pow; maxi[i] = r[i].maxi; outers[i] = r[i].outers;
    }
    *count = (int)r.size();
  });
}

int ora_xs_updt_at(void* h, double bcon) { Ora* o = (Ora*)h; return guard(o, [&] { xs_updt_at(*o, bcon); }); }

int ora_outer(void* h, int adj, int popt, int max_outers) {
  Ora* o = (Ora*)h;
  return guard(o, [&] { outer(*o, adj != 0, popt, max_outers); });
}

int ora_powdis(void* h, double* p) { Ora* o = (Ora*)h; return guard(o, [&] { powdis(*o, p); }); }
int ora_matrix_setup(void* h, int opt) { Ora* o = (Ora*)h; return guard(o, [&] { matrix_setup(*o, opt); }); }
int ora_nodal_upd(void* h, int nmode) { Ora* o = (Ora*)h; return guard(o, [&] { nodal_upd(*o, nmode); }); }

// One group solve: bs from TSrc/TSrcAd with the current state, then bicg.
int ora_group_solve(void* h, int g, int adj, double* bs_out) {
  Ora* o = (Ora*)h;
  return guard(o, [&] {
    std::vector<double> bs(o->nnod);
    tsrc(*o, g, o->Ke, bs, adj != 0);
    if (bs_out) std::copy(bs.begin(), bs.end(), bs_out);
    bicg(*o, o->nin, g, bs, &o->f0[(size_t)o->nnod * (g - 1)]);
  });
}

int ora_bicg(void* h, int g, int imax, const double* b, double* x) {
  Ora* o = (Ora*)h;
  return guard(o, [&] {
    std::vector<double> bv(b, b + o->nnod);
    bicg(*o, imax, g, bv, x);
  });
}

// The CMFD matrix in a fixed 7-slot row form [z-,y-,x-,diag,x+,y+,z+],
// zeros where the reference has no element.  out: (7, nnod, ng)
int ora_get_matrix7(void* h, double* out) {
  Ora* o = (Ora*)h;
  return guard(o, [&] {
    for (int g = 1; g <= o->ng; ++g)
      for (int n = 1; n <= o->nnod; ++n) {
        int i = o->ix[n - 1], j = o->iy[n - 1], k = o->iz[n - 1];
        bool has[7] = {k != 1, j != o->xsmin[i - 1], i != o->ysmin[j - 1], true, i != o->ysmax[j - 1],
                       j != o->xsmax[i - 1], k != o->nzz};
        int rec = 0;
        for (int c = 0; c < 7; ++c) {
          double v = 0.0;
          if (has[c]) v = o->AE(++rec, n, g);
          out[c + 7 * ((n - 1) + (size_t)o->nnod * (g - 1))] = v;
        }
      }
  });
}

// af, sigrp: (nnod, ng); sigrp NULL for the oracle's own sigr
int ora_reactivity(void* h, const double* af, const double* sigrp, double* rho) {
  Ora* o = (Ora*)h;
  return guard(o, [&] { *rho = reactivity(*o, af, sigrp ? sigrp : o->sigr.data()); });
}

int ora_calc_beta(void* h, const double* af, int nf, const double* ibeta, double* beta) {
  Ora* o = (Ora*)h;
  return guard(o, [&] { *beta = calc_beta(*o, af, nf, ibeta); });
}

int ora_asmpow(void* h, const double* fn, double* fasm, int* imax, int* jmax) {
  Ora* o = (Ora*)h;
  return guard(o, [&] { asmpow(*o, fn, fasm, imax, jmax); });
}

int ora_axipow(void* h, const double* fn, double* faxi, int* kmax) {
  Ora* o = (Ora*)h;
  return guard(o, [&] { axipow(*o, fn, faxi, kmax); });
}

// f: (nnod, ng) flux, NULL for the oracle's own f0; norm <= 0: not given
int ora_asmflux(void* h, const double* f, double norm, double* fasm, int* negf) {
  Ora* o = (Ora*)h;
  return guard(o, [&] { asmflux(*o, f ? f : o->f0.data(), norm > 0, norm, fasm, negf); });
}

int ora_get_int(void* h, const char* name) {
  Ora* o = (Ora*)h;
  std::string s(name);
  if (s == "ng") return o->ng;
  if (s == "nmat") return o->nmat;
  if (s == "nnod") return o->nnod;
  if (s == "nxx") return o->nxx;
  if (s == "nyy") return o->nyy;
  if (s == "nzz") return o->nzz;
  if (s == "nx") return o->nx;
  if (s == "ny") return o->ny;
  if (s == "nz") return o->nz;
  if (s == "nin") return o->nin;
  if (s == "nout") return o->nout;
  if (s == "nac") return o->nac;
  if (s == "nupd") return o->nupd;
  if (s == "xeast") return o->xeast;
  if (s == "xwest") return o->xwest;
  if (s == "ynorth") return o->ynorth;
  if (s == "ysouth") return o->ysouth;
  if (s == "zbott") return o->zbott;
  if (s == "ztop") return o->ztop;
  if (s == "kern") return o->kern == " FDM" ? 0 : (o->kern == " PNM" ? 1 : 2);
  if (s == "adjoint") return o->mode == "ADJOINT" ? 1 : 0;
  if (s == "bcsearch") return o->mode == "BCSEARCH" ? 1 : 0;
  if (s == "rodeject") return o->mode == "RODEJECT" ? 1 : 0;
  if (s == "im") return o->im;
  if (s == "jm") return o->jm;
  if (s == "km") return o->km;
  if (s == "outers") return o->last_outers;
  if (s == "trace_len") return (int)o->trace.size();
  if (s == "badf") return o->badf ? 1 : 0;
  return -1;
}

double ora_get_double(void* h, const char* name) {
  Ora* o = (Ora*)h;
  std::string s(name);
  if (s == "Ke") return o->Ke;
  if (s == "ndmax") return o->ndmax;
  if (s == "serc") return o->serc;
  if (s == "ferc") return o->ferc;
  if (s == "ser") return o->last_ser;
  if (s == "fer") return o->last_fer;
  if (s == "t_cmfd") return o->t_cmfd;
  if (s == "t_nodal") return o->t_nodal;
  return NAN;
}

int ora_set_double(void* h, const char* name, double v) {
  Ora* o = (Ora*)h;
  std::string s(name);
  if (s == "Ke") { o->Ke = v; return 0; }
  if (s == "ndmax") { o->ndmax = v; return 0; }
  if (s == "serc") { o->serc = v; return 0; }
  if (s == "ferc") { o->ferc = v; return 0; }
  return -1;
}

int ora_set_int(void* h, const char* name, int v) {
  Ora* o = (Ora*)h;
  std::string s(name);
  if (s == "nout") { o->nout = v; return 0; }
  if (s == "nin") { o->nin = v; return 0; }
  if (s == "nac") { o->nac = v; return 0; }
  if (s == "nupd") { o->nupd = v; return 0; }
  return -1;
}

long ora_array_len(void* h, const char* name) {
  Ora* o = (Ora*)h;
  if (auto* v = dvec(o, name)) return (long)v->size();
  if (auto* v = ivec(o, name)) return (long)v->size();
  return -1;
}

int ora_get_array(void* h, const char* name, double* out) {
  Ora* o = (Ora*)h;
  auto* v = dvec(o, name);
  if (!v) return -1;
  std::copy(v->begin(), v->end(), out);
  return 0;
}

int ora_set_array(void* h, const char* name, const double* in) {
  Ora* o = (Ora*)h;
  auto* v = dvec(o, name);
  if (!v) return -1;
  std::copy(in, in + v->size(), v->begin());
  return 0;
}

int ora_get_iarray(void* h, const char* name, int* out) {
  Ora* o = (Ora*)h;
  auto* v = ivec(o, name);
  if (!v) return -1;
  std::copy(v->begin(), v->end(), out);
  return 0;
}

// trace: p, k, ser, fer, extrapolated, nodal, ndmax, im, jm, km
int ora_get_trace(void* h, int* ip, double* k, double* ser, double* fer, int* flags, double* ndmax, int* loc) {
  Ora* o = (Ora*)h;
  for (size_t t = 0; t < o->trace.size(); ++t) {
    const TraceRec& r = o->trace[t];
    ip[t] = r.p; k[t] = r.k; ser[t] = r.ser; fer[t] = r.fer;
    flags[t] = r.extrapolated | (r.nodal << 1);
    ndmax[t] = r.ndmax;
    loc[3 * t] = r.im; loc[3 * t + 1] = r.jm; loc[3 * t + 2] = r.km;
  }
  return (int)o->trace.size();
}

// Reset the solver state so that the next outer call starts cold (f0 = 1,
// k = 1, dn = 0), as a fresh reference process would.
void ora_reset(void* h) {
  Ora* o = (Ora*)h;
  o->coup_first = true; o->outer_first = true; o->outer_ad_first = true;
  o->ndmax = 0.0; o->im = o->jm = o->km = 0;
  o->f0.clear(); o->fs0.clear(); o->s0.clear();
  o->t_cmfd = o->t_nodal = 0.0;
}

}  // extern "C"
