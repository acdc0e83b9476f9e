/*
 * fe_oracle.c -- CPU restatement of the reference's force-engine hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline; never the
 * product path).  Each function restates one reference routine in the same
 * floating-point operation order; the citation is on each function.  Built
 * with -O2 -ffp-contract=off and no fast-math it reproduces a strict build of
 * the reference bit for bit (pinned by tests/test_oracle_pin.py against the
 * reference itself, and by tests/golden fixtures made from it).
 *
 * Physical constants are the reference's (defines.h:62-75).  QFACTOR in the
 * reference is an unparenthesised macro, so `a*b*QFACTOR` evaluates as
 * ((((a*b)*ELEC)*ELEQ)*ELEQ)*NA)*1e-3; QF() below keeps that order.
 */
#include "fe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "fe_fft.h"

#define PI_ 3.141592653589793238462643383
#define KB_ 1.380662E-23
#define NA_ 6.022045E23
#define AU_ 1.6605655E-27
#define ELEC_ 8.987551789e19
#define ELEQ_ 1.602176462e-19
#define E14FAC_ 0.4
#define QF(x) (((((x) * ELEC_) * ELEQ_) * ELEQ_) * NA_ * 1.0E-3)

/* The reference links its own erfc (ewald.c:817-836), which overrides libm's
 * in every EWALD build: the Chebyshev fit "erfcc" of Numerical Recipes
 * (Press et al., 2nd ed., sec. 6.2), fractional error < 1.2e-7.  Restated
 * here with the same evaluation order. */
static double ref_erfc(double x) {
  double z = fabs(x);
  double t = 1.0 / (1.0 + 0.5 * z);
  double v = t * exp(-z * z + -1.26551223 +
                     t * (1.00002368 +
                     t * (0.37409196 +
                     t * (0.09678418 +
                     t * (-0.18628806 +
                     t * (0.27886807 +
                     t * (-1.13520398 +
                     t * (1.48851587 +
                     t * (-0.82215223 + t * 0.17087277)))))))));
  if (x < 0) return 2.0 - v;
  return v;
}

void or_setlj(int ntypes, const double *eps_kcal, const double *rmin_half,
              double *lj_eps, double *lj_sig) {
  /* setlj.c:181-191 */
  for (int a = 0; a < ntypes; a++)
    for (int b = 0; b < ntypes; b++) {
      lj_eps[a * ntypes + b] = 4.184 * sqrt(eps_kcal[a] * eps_kcal[b]);
      lj_sig[a * ntypes + b] = 0.5 * (2.0 * rmin_half[a] + 2.0 * rmin_half[b]);
    }
}

/* ------------------------------------------------------------------------ */
/* exclusion lookup: the reference hashes xint (setlj.c:211-247) and, for a
 * listed pair, scans the chain with the LAST matching entry winning
 * (nblist.c:156-174).  Here: per-atom partner lists in xint order. */
typedef struct {
  int *start; /* n+1 */
  int *partner;
  int *flag;
} xtab;

static void xtab_build(const or_system *s, xtab *t) {
  int n = s->n;
  t->start = (int *)calloc((size_t)n + 1, sizeof(int));
  t->partner = (int *)malloc(sizeof(int) * (size_t)(2 * s->nexcl + 1));
  t->flag = (int *)malloc(sizeof(int) * (size_t)(2 * s->nexcl + 1));
  for (int i = 0; i < s->nexcl; i++) {
    t->start[s->excl_ab[2 * i] + 1]++;
    t->start[s->excl_ab[2 * i + 1] + 1]++;
  }
  for (int i = 0; i < n; i++) t->start[i + 1] += t->start[i];
  int *fill = (int *)calloc((size_t)n, sizeof(int));
  for (int i = 0; i < s->nexcl; i++) {
    int a = s->excl_ab[2 * i], b = s->excl_ab[2 * i + 1];
    int pa = t->start[a] + fill[a]++;
    t->partner[pa] = b;
    t->flag[pa] = s->excl_flag[i];
    int pb = t->start[b] + fill[b]++;
    t->partner[pb] = a;
    t->flag[pb] = s->excl_flag[i];
  }
  free(fill);
}

static int xtab_flag(const xtab *t, int a, int b) {
  int f = 0;
  for (int p = t->start[a]; p < t->start[a + 1]; p++)
    if (t->partner[p] == b) f = t->flag[p];
  return f;
}

static void xtab_free(xtab *t) {
  free(t->start);
  free(t->partner);
  free(t->flag);
}

/* ------------------------------------------------------------------------ */
int64_t or_nblist(const or_system *s, const double *pos, int *cnt, int *idx,
                  int *flag, int64_t cap, int *cnt_ew, int *idx_ew,
                  int *flag_ew, int64_t cap_ew) {
  /* nblist.c:32-325, EWALD + STYPE branch, no CLIST */
  double lx = s->L[0], ly = s->L[1], lz = s->L[2];
  double hx = lx / 2.0, hy = ly / 2.0, hz = lz / 2.0;
  double rcut = s->rclist;
  double rcut2 = s->rclist * s->rclist;
  double rcut_ew = s->rclist_ew;
  double rcut2_ew = rcut_ew * rcut_ew;
  int ns = s->n;
  xtab t;
  xtab_build(s, &t);
  int64_t p = 0, pe = 0;
  for (int i = 0; i < ns; i++) {
    if (cnt) cnt[i] = 0;
    if (cnt_ew) cnt_ew[i] = 0;
  }
  for (int a = 0; a < ns - 1; a++) {
    double ax = pos[3 * a], ay = pos[3 * a + 1], az = pos[3 * a + 2];
    for (int b = a + 1; b < ns; b++) {
      double dx = fabs(ax - pos[3 * b]);
      if (dx > hx) dx -= lx;
      if (dx > rcut) continue;
      double dy = fabs(ay - pos[3 * b + 1]);
      if (dy > hy) dy -= ly;
      if (dy > rcut) continue;
      double dz = fabs(az - pos[3 * b + 2]);
      if (dz > hz) dz -= lz;
      if (dz > rcut) continue;
      double dr2 = dx * dx + dy * dy + dz * dz;
      if (dr2 < rcut2_ew) {
        int xf = s->nexcl ? xtab_flag(&t, a, b) : 0;
        if (cnt_ew) {
          if (pe >= cap_ew) { xtab_free(&t); return -1; }
          idx_ew[pe] = b;
          if (flag_ew) flag_ew[pe] = xf;
          pe++;
          cnt_ew[a]++;
        }
        if (dr2 < rcut2 && cnt) {
          if (p >= cap) { xtab_free(&t); return -1; }
          idx[p] = b;
          if (flag) flag[p] = xf;
          p++;
          cnt[a]++;
        }
      }
    }
  }
  xtab_free(&t);
  return p;
}

/* ------------------------------------------------------------------------ */
void or_cnonbond_pairs(const or_system *s, const double *pos, const int *cnt,
                       const int *idx, const int *flag, double *ff,
                       double e5[5]) {
  /* cnonbond_nblist.c:51-523 (SPME + STYPE, CHARMM LJ form) */
  double enonbond = 0.0, enonbonds = 0.0;
  double kappa = s->kappa;
  double kpi = 1.0 * kappa / sqrt(PI_);
  double eewald_real = 0.0, eewald_reals = 0.0, eewald_intra = 0.0;
  double rc = s->rc;
  double rc2 = rc * rc; /* box[k].rc2, read_config.c:329 */
  double lx = s->L[0], ly = s->L[1], lz = s->L[2];
  double hx = lx / 2.0, hy = ly / 2.0, hz = lz / 2.0;
  int nt = s->ntypes;
  /* optional CHARMM switch (Brooks et al. 1983), absent in the reference */
  double ron2 = s->r_switch > 0.0 ? s->r_switch * s->r_switch : 0.0;
  double sw_den = 0.0;
  if (ron2 > 0.0) sw_den = (rc2 - ron2) * (rc2 - ron2) * (rc2 - ron2);
  int64_t off = 0;
  for (int a = 0; a < s->n - 1; a++) {
    double fxa = 0.0, fya = 0.0, fza = 0.0;
    double ax = pos[3 * a], ay = pos[3 * a + 1], az = pos[3 * a + 2];
    for (int bb = 0; bb < cnt[a]; bb++) {
      int b = idx[off + bb];
      double dx = ax - pos[3 * b];
      double dy = ay - pos[3 * b + 1];
      double dz = az - pos[3 * b + 2];
      if (dx > hx) dx -= lx;
      else if (dx < -hx) dx += lx;
      if (dy > hy) dy -= ly;
      else if (dy < -hy) dy += ly;
      if (dz > hz) dz -= lz;
      else if (dz < -hz) dz += lz;
      double dr2 = dx * dx + dy * dy + dz * dz;
      if (dr2 > rc2) continue;
      int ta = s->type[a], tb = s->type[b];
      int xflag = flag ? flag[off + bb] : 0;
      double sig = s->lj_sig[ta * nt + tb];
      double eps = s->lj_eps[ta * nt + tb];
      double qq = QF(s->q[a] * s->q[b]);
      double qqab = qq;
      if (xflag) {
        if (xflag != 4) {
          sig = 0.0;
          eps = 0.0;
          qq = 0.0;
        } else
          qq *= E14FAC_;
      }
      double force = 0.0;
      if ((eps * sig) != 0.0) {
        double sr2 = (sig * sig) / dr2;
        double sr6 = sr2 * sr2 * sr2;
        double sr12 = sr6 * sr6;
        double sr2s = (sig * sig) / rc2;
        double sr6s = sr2s * sr2s * sr2s;
        double sr12s = sr6s * sr6s;
        double flj = (12.0 * eps / dr2) * (sr12 - sr6);
        double elj = eps * (sr12 - 2.0 * sr6);
        if (s->lj_form == 2) { /* the BGO build, cnonbond_nblist.c:294-307 */
          double sr10 = sr6 * sr2 * sr2;
          double sr10s = sr6s * sr2s * sr2s;
          force = eps / dr2 * (156.0 * sr12 - 180.0 * sr10 + 24.0 * sr6);
          enonbond += eps * (13.0 * sr12 - 18.0 * sr10 + 4.0 * sr6);
          enonbonds += eps * (13.0 * sr12s - 18.0 * sr10s + 4.0 * sr6s);
        } else if (ron2 > 0.0) {
          if (dr2 > ron2) {
            double c = rc2 - dr2;
            double sw = c * c * (rc2 + 2.0 * dr2 - 3.0 * ron2) / sw_den;
            double dsw = 12.0 * c * (dr2 - ron2) / sw_den; /* = -2 dS/d(r^2) */
            flj = flj * sw + elj * dsw;
            elj = elj * sw;
          }
          force = flj;
          enonbond += elj;
        } else {
          force = flj;
          enonbond += elj;
          enonbonds += eps * (sr12s - 2.0 * sr6s);
        }
      }
      double dr = sqrt(dr2);
      double dri = 1.0 / dr;
      double kr = kappa * dr;
      double erfckr = ref_erfc(kr);
      double kpidrexpkr2 = 2.0 * kpi * dr * exp(-kr * kr);
      qq /= s->epsRF;
      if (qq != 0.0) {
        eewald_real += qq * erfckr * dri;
        eewald_reals += qq * ref_erfc(kappa * rc) / rc;
        force += (qq * dri / dr2) * (erfckr + kpidrexpkr2);
      }
      if (xflag) {
        if (xflag == 4) qqab *= (1.0 - E14FAC_);
        eewald_intra += qqab * (1.0 - erfckr) * dri;
        force -= (qqab * dri / dr2) * ((1.0 - erfckr) - kpidrexpkr2);
      }
      if (force != 0.0) {
        double fx = force * dx;
        fxa += fx;
        ff[3 * b] -= fx;
        double fy = force * dy;
        fya += fy;
        ff[3 * b + 1] -= fy;
        double fz = force * dz;
        fza += fz;
        ff[3 * b + 2] -= fz;
      }
    }
    off += cnt[a];
    ff[3 * a] += fxa;
    ff[3 * a + 1] += fya;
    ff[3 * a + 2] += fza;
  }
  e5[0] = enonbond;
  e5[1] = enonbonds;
  e5[2] = eewald_real;
  e5[3] = eewald_reals;
  e5[4] = eewald_intra;
}

/* ------------------------------------------------------------------------ */
static void fillspline(int ORDER, double w, double *array, double *darray) {
  /* pme_spline.c:10-49 */
  for (int i = 3; i <= ORDER; i++) array[i] = 0.0;
  array[2] = w;
  array[1] = 1.0 - w;
  array[0] = 0.0;
  for (int i = 3; i <= ORDER - 1; i++) {
    double div = (double)(1.0 / (i - 1));
    array[i] = div * w * array[i - 1];
    double di = (double)(i);
    for (int j = 1; j <= (i - 2); j++) {
      double dj = (double)(j);
      array[i - j] = div * ((w + dj) * array[i - j - 1] + (di - dj - w) * array[i - j]);
    }
    array[1] *= div * (1.0 - w);
  }
  darray[0] = 0.0;
  darray[1] = -array[1];
  for (int i = 2; i <= ORDER; i++) darray[i] = array[i - 1] - array[i];
  int kk = ORDER;
  double div = (double)(1.0 / (kk - 1));
  array[kk] = div * w * array[kk - 1];
  double dkk = (double)(kk);
  for (int i = 1; i <= (kk - 2); i++) {
    double di = (double)(i);
    array[kk - i] = div * ((w + di) * array[kk - i - 1] + (dkk - di - w) * array[kk - i]);
  }
  array[1] *= div * (1.0 - w);
}

void or_fillspline(int order, double w, double *array, double *darray) {
  fillspline(order, w, array, darray);
}

/* drift.c:21-66: net momentum / n subtracted as (P / n) / m_i */
void or_drift(const or_system *s, double *vv) {
  double vvx = 0.0, vvy = 0.0, vvz = 0.0;
  for (int i = 0; i < s->n; i++) {
    vvx += s->mass[i] * vv[3 * i];
    vvy += s->mass[i] * vv[3 * i + 1];
    vvz += s->mass[i] * vv[3 * i + 2];
  }
  vvx /= (1.0 * s->n);
  vvy /= (1.0 * s->n);
  vvz /= (1.0 * s->n);
  for (int i = 0; i < s->n; i++) {
    double imass = 1.0 / s->mass[i];
    vv[3 * i] -= vvx * imass;
    vv[3 * i + 1] -= vvy * imass;
    vv[3 * i + 2] -= vvz * imass;
  }
}

static void dftmod(double *bmod, const double *barr, int grid) {
  /* pme_setup.c:110-130 */
  double twopi = 2.0 * PI_;
  for (int i = 1; i <= grid; i++) {
    double sum1 = 0.0, sum2 = 0.0;
    for (int j = 1; j <= grid; j++) {
      double arg = twopi * (i - 1) * (j - 1) / grid;
      sum1 += barr[j] * cos(arg);
      sum2 += barr[j] * sin(arg);
    }
    bmod[i] = sum1 * sum1 + sum2 * sum2;
  }
}

void or_pme_bspline(const or_system *s, double *bx, double *by, double *bz) {
  /* pme_setup.c:86-107 */
  int ORDER = s->order;
  double mn[64], dmn[64];
  fillspline(ORDER, 0.0, mn, dmn);
  int gmax = s->grid[0];
  if (s->grid[1] > gmax) gmax = s->grid[1];
  if (s->grid[2] > gmax) gmax = s->grid[2];
  int ngrid = gmax + 1;
  double *arr = (double *)calloc((size_t)ngrid + 6, sizeof(double));
  for (int i = 2; i <= ORDER + 1; i++) arr[i] = mn[i - 1];
  dftmod(bx, arr, s->grid[0]);
  dftmod(by, arr, s->grid[1]);
  dftmod(bz, arr, s->grid[2]);
  free(arr);
}

typedef struct {
  double *ss;  /* 3n */
  double *mm;  /* n*(ORDER+1)*3, [i][n][axis] */
  double *dm;
} splines;

static void spline_fill(const or_system *s, const double *pos, splines *sp) {
  /* pme_qgrid.c:26-70 */
  int ORDER = s->order;
  int n = s->n;
  double blx = s->L[0], bly = s->L[1], blz = s->L[2];
  sp->ss = (double *)malloc(sizeof(double) * 3 * (size_t)n);
  sp->mm = (double *)calloc((size_t)n * (ORDER + 1) * 3, sizeof(double));
  sp->dm = (double *)calloc((size_t)n * (ORDER + 1) * 3, sizeof(double));
  for (int i = 0; i < n; i++) {
    double qx = pos[3 * i] / blx;
    double qy = pos[3 * i + 1] / bly;
    double qz = pos[3 * i + 2] / blz;
    sp->ss[3 * i] = s->grid[0] * (qx + 0.5);
    sp->ss[3 * i + 1] = s->grid[1] * (qy + 0.5);
    sp->ss[3 * i + 2] = s->grid[2] * (qz + 0.5);
  }
  double mn[64], dmn[64];
  for (int i = 0; i < n; i++)
    for (int ax = 0; ax < 3; ax++) {
      double sv = sp->ss[3 * i + ax];
      double w = sv - (int)(sv);
      fillspline(ORDER, w, mn, dmn);
      for (int m = 1; m <= ORDER; m++) {
        sp->mm[((size_t)i * (ORDER + 1) + m) * 3 + ax] = mn[m];
        sp->dm[((size_t)i * (ORDER + 1) + m) * 3 + ax] = dmn[m];
      }
    }
}

static void splines_free(splines *sp) {
  free(sp->ss);
  free(sp->mm);
  free(sp->dm);
}

static void spread(const or_system *s, const splines *sp, double *cgrid) {
  /* pme_qgrid.c:74-117; cgrid is complex (2 doubles per point) */
  int ORDER = s->order;
  int GX = s->grid[0], GY = s->grid[1], GZ = s->grid[2];
  long ngrid = (long)GX * GY * GZ;
  for (long i = 0; i < ngrid; i++) {
    cgrid[2 * i] = 0.0;
    cgrid[2 * i + 1] = 0.0;
  }
  for (int i = 0; i < s->n; i++) {
    double qq = s->q[i];
    int xxo = (int)(sp->ss[3 * i]) - ORDER;
    int yyo = (int)(sp->ss[3 * i + 1]) - ORDER;
    int zzo = (int)(sp->ss[3 * i + 2]) - ORDER;
    int xo = xxo;
    for (int xi = 1; xi <= ORDER; xi++) {
      xo++;
      int x = xo + (xo < 0 ? GX : 0);
      double mxi = sp->mm[((size_t)i * (ORDER + 1) + xi) * 3 + 0];
      int yo = yyo;
      for (int yi = 1; yi <= ORDER; yi++) {
        yo++;
        int y = yo + (yo < 0 ? GY : 0);
        double myi = sp->mm[((size_t)i * (ORDER + 1) + yi) * 3 + 1];
        int zo = zzo;
        for (int zi = 1; zi <= ORDER; zi++) {
          zo++;
          int z = zo + (zo < 0 ? GZ : 0);
          double mzi = sp->mm[((size_t)i * (ORDER + 1) + zi) * 3 + 2];
          long index = (long)z + (long)y * GZ + (long)x * GY * GZ;
          cgrid[2 * index] += mxi * myi * mzi * qq;
        }
      }
    }
  }
}

void or_charge_grid(const or_system *s, const double *pos, double *grid) {
  splines sp;
  spline_fill(s, pos, &sp);
  long ng = (long)s->grid[0] * s->grid[1] * s->grid[2];
  double *c = (double *)malloc(sizeof(double) * 2 * (size_t)ng);
  spread(s, &sp, c);
  for (long i = 0; i < ng; i++) grid[i] = c[2 * i];
  free(c);
  splines_free(&sp);
}

void or_pme_calc(const or_system *s, const double *pos, double sewald,
                 double *ff, double e3[3]) {
  /* pme_calc.c:18-119 */
  int ORDER = s->order;
  int GX = s->grid[0], GY = s->grid[1], GZ = s->grid[2];
  double blx = s->L[0], bly = s->L[1], blz = s->L[2];
  double vol = blx * bly * blz;
  double kap = s->kappa;
  double fac = PI_ * PI_ / kap / kap;
  double enrec = 0.0;
  long ngrid = (long)GX * GY * GZ;
  long ggyz = (long)GY * GZ;
  double *bx = (double *)calloc((size_t)GX + 2, sizeof(double));
  double *by = (double *)calloc((size_t)GY + 2, sizeof(double));
  double *bz = (double *)calloc((size_t)GZ + 2, sizeof(double));
  or_pme_bspline(s, bx, by, bz);
  splines sp;
  spline_fill(s, pos, &sp);
  double *q = (double *)malloc(sizeof(double) * 2 * (size_t)ngrid);
  spread(s, &sp, q);
  fe_fft3d(q, GX, GY, GZ, +1); /* FFTW_BACKWARD */
  for (long ind = 1; ind < ngrid; ind++) {
    int k1 = (int)(ind / ggyz);
    long knd = ind - k1 * ggyz;
    int k2 = (int)(knd / GZ);
    int k3 = (int)(knd - (long)k2 * GZ);
    int mx = k1 - (k1 > GX / 2 ? GX : 0);
    int my = k2 - (k2 > GY / 2 ? GY : 0);
    int mz = k3 - (k3 > GZ / 2 ? GZ : 0);
    double mhatx = mx / blx;
    double mhaty = my / bly;
    double mhatz = mz / blz;
    double mm = mhatx * mhatx + mhaty * mhaty + mhatz * mhatz;
    double bb = bx[k1 + 1] * by[k2 + 1] * bz[k3 + 1];
    double den = PI_ * vol * mm * bb;
    double eterm = exp(-fac * mm) / den;
    long index = (long)k3 + (long)k2 * GZ + (long)k1 * GY * GZ;
    double qr = q[2 * index];
    double qi = q[2 * index + 1];
    double struc2 = qr * qr + qi * qi;
    enrec += eterm * struc2;
    q[2 * index] *= eterm;
    q[2 * index + 1] *= eterm;
  }
  double fan = 0.5 * ELEC_ * ELEQ_ * ELEQ_ * NA_ * 1.0E-3 / s->epsRF;
  e3[0] = enrec * fan;
  e3[1] = sewald;
  e3[2] = e3[0] - e3[1];
  fe_fft3d(q, GX, GY, GZ, -1); /* FFTW_FORWARD */

  /* pme_force, pme_calc.c:122-279 (the reference's separate block for the
   * last atom performs the same arithmetic as the loop body) */
  double sumx = 0.0, sumy = 0.0, sumz = 0.0;
  int nsite = s->n;
  double *fi = (double *)malloc(sizeof(double) * 3 * (size_t)nsite);
  for (int i = 0; i < nsite; i++) {
    double fxi = 0.0, fyi = 0.0, fzi = 0.0;
    int xxo = (int)(sp.ss[3 * i]) - ORDER;
    int yyo = (int)(sp.ss[3 * i + 1]) - ORDER;
    int zzo = (int)(sp.ss[3 * i + 2]) - ORDER;
    int xo = xxo;
    for (int xi = 1; xi <= ORDER; xi++) {
      xo++;
      int x = xo + (xo < 0 ? GX : 0);
      double mxi = sp.mm[((size_t)i * (ORDER + 1) + xi) * 3 + 0];
      double dmxi = sp.dm[((size_t)i * (ORDER + 1) + xi) * 3 + 0];
      int yo = yyo;
      for (int yi = 1; yi <= ORDER; yi++) {
        yo++;
        int y = yo + (yo < 0 ? GY : 0);
        double myi = sp.mm[((size_t)i * (ORDER + 1) + yi) * 3 + 1];
        double dmyi = sp.dm[((size_t)i * (ORDER + 1) + yi) * 3 + 1];
        int zo = zzo;
        for (int zi = 1; zi <= ORDER; zi++) {
          zo++;
          int z = zo + (zo < 0 ? GZ : 0);
          double mzi = sp.mm[((size_t)i * (ORDER + 1) + zi) * 3 + 2];
          double dmzi = sp.dm[((size_t)i * (ORDER + 1) + zi) * 3 + 2];
          long index = (long)z + (long)y * GZ + (long)x * GY * GZ;
          double term = q[2 * index];
          fxi -= dmxi * myi * mzi * term;
          fyi -= mxi * dmyi * mzi * term;
          fzi -= mxi * myi * dmzi * term;
        }
      }
    }
    double qq = s->q[i];
    double facq = QF(qq) / s->epsRF;
    fxi *= facq * GX / blx;
    fyi *= facq * GY / bly;
    fzi *= facq * GZ / blz;
    ff[3 * i] += fxi;
    ff[3 * i + 1] += fyi;
    ff[3 * i + 2] += fzi;
    sumx += fxi;
    sumy += fyi;
    sumz += fzi;
  }
  sumx /= (double)(nsite);
  sumy /= (double)(nsite);
  sumz /= (double)(nsite);
  for (int i = 0; i < nsite; i++) {
    ff[3 * i] -= sumx;
    ff[3 * i + 1] -= sumy;
    ff[3 * i + 2] -= sumz;
  }
  free(fi);
  free(q);
  splines_free(&sp);
  free(bx);
  free(by);
  free(bz);
}

double or_ewald_self(const or_system *s) {
  /* ewald.c:61,172-178 */
  double fconv = (ELEC_ * ELEQ_ * ELEQ_ * NA_ * 0.001) / s->epsRF;
  double vs = 0.0;
  for (int i = 0; i < s->n; i++) vs += s->q[i] * s->q[i];
  vs *= s->kappa / sqrt(PI_);
  return vs * fconv;
}

/* ------------------------------------------------------------------------ */
double or_cbond(const or_system *s, const double *pos, double *ff) {
  /* cbond.c:27-180 */
  double ebond = 0.0;
  double lx = s->L[0], ly = s->L[1], lz = s->L[2];
  double hx = lx / 2.0, hy = ly / 2.0, hz = lz / 2.0;
  for (int i = 0; i < s->nbond; i++) {
    int ia = s->bond_ab[2 * i], ib = s->bond_ab[2 * i + 1];
    double dx = pos[3 * ib] - pos[3 * ia];
    double dy = pos[3 * ib + 1] - pos[3 * ia + 1];
    double dz = pos[3 * ib + 2] - pos[3 * ia + 2];
    if (dx > hx) dx -= lx;
    else if (dx < -hx) dx += lx;
    if (dy > hy) dy -= ly;
    else if (dy < -hy) dy += ly;
    if (dz > hz) dz -= lz;
    else if (dz < -hz) dz += lz;
    double drr = dx * dx + dy * dy + dz * dz;
    double dr = sqrt(drr);
    double dri = 1.0 / dr;
    double rr = dr - s->bond_req[i];
    double fr = -s->bond_k[i] * rr * 2.0;
    ebond += -(fr * rr * 0.5);
    double fx = fr * dri * dx;
    double fy = fr * dri * dy;
    double fz = fr * dri * dz;
    ff[3 * ia] -= fx;
    ff[3 * ia + 1] -= fy;
    ff[3 * ia + 2] -= fz;
    ff[3 * ib] += fx;
    ff[3 * ib + 1] += fy;
    ff[3 * ib + 2] += fz;
  }
  return ebond;
}

double or_cbend(const or_system *s, const double *pos, double *ff) {
  /* cbend.c:24-218 */
  double ebend = 0.0;
  double lx = s->L[0], ly = s->L[1], lz = s->L[2];
  double hx = lx / 2.0, hy = ly / 2.0, hz = lz / 2.0;
  for (int i = 0; i < s->nbend; i++) {
    int ia = s->bend_abc[3 * i], ib = s->bend_abc[3 * i + 1], ic = s->bend_abc[3 * i + 2];
    double dax = pos[3 * ia] - pos[3 * ib];
    double day = pos[3 * ia + 1] - pos[3 * ib + 1];
    double daz = pos[3 * ia + 2] - pos[3 * ib + 2];
    double dcx = pos[3 * ic] - pos[3 * ib];
    double dcy = pos[3 * ic + 1] - pos[3 * ib + 1];
    double dcz = pos[3 * ic + 2] - pos[3 * ib + 2];
    if (dax > hx) dax -= lx;
    else if (dax < -hx) dax += lx;
    if (day > hy) day -= ly;
    else if (day < -hy) day += ly;
    if (daz > hz) daz -= lz;
    else if (daz < -hz) daz += lz;
    if (dcx > hx) dcx -= lx;
    else if (dcx < -hx) dcx += lx;
    if (dcy > hy) dcy -= ly;
    else if (dcy < -hy) dcy += ly;
    if (dcz > hz) dcz -= lz;
    else if (dcz < -hz) dcz += lz;
    double drai = 1.0 / sqrt(dax * dax + day * day + daz * daz);
    double erax = dax * drai, eray = day * drai, eraz = daz * drai;
    double drci = 1.0 / sqrt(dcx * dcx + dcy * dcy + dcz * dcz);
    double ercx = dcx * drci, ercy = dcy * drci, ercz = dcz * drci;
    double cosphi = erax * ercx + eray * ercy + eraz * ercz;
    double phi = acos(cosphi);
    double isinphi = 1.0 / sqrt(1.0 - cosphi * cosphi);
    double rr = phi - s->bend_theta0[i];
    double fr = -s->bend_k[i] * rr * 2.0;
    ebend += -fr * rr * 0.5;
    double irasin = drai * isinphi * fr;
    double ircsin = drci * isinphi * fr;
    double fxa = (erax * cosphi - ercx) * irasin;
    double fya = (eray * cosphi - ercy) * irasin;
    double fza = (eraz * cosphi - ercz) * irasin;
    double fxc = (ercx * cosphi - erax) * ircsin;
    double fyc = (ercy * cosphi - eray) * ircsin;
    double fzc = (ercz * cosphi - eraz) * ircsin;
    ff[3 * ia] += fxa;
    ff[3 * ia + 1] += fya;
    ff[3 * ia + 2] += fza;
    ff[3 * ib] += -(fxa + fxc);
    ff[3 * ib + 1] += -(fya + fyc);
    ff[3 * ib + 2] += -(fza + fzc);
    ff[3 * ic] += fxc;
    ff[3 * ic + 1] += fyc;
    ff[3 * ic + 2] += fzc;
  }
  return ebend;
}

/* ------------------------------------------------------------------------ */
/* minimum image of one separation, the branch form of cbond.c / ctorsion.c */
static void or_min_image(const or_system *s, double *d) {
  for (int c = 0; c < 3; c++) {
    double l = s->L[c], h = l / 2.0;
    if (d[c] > h) d[c] -= l;
    else if (d[c] < -h) d[c] += l;
  }
}

double or_curey(const or_system *s, const double *pos, int nurey, const int *ab,
                const double *seq, const double *k, double *ff) {
  /* curey.c:37-106: E = k (r - Seq)^2 on the 1-3 distance */
  double eurey = 0.0;
  for (int i = 0; i < nurey; i++) {
    int ia = ab[2 * i], ib = ab[2 * i + 1];
    double d[3];
    for (int c = 0; c < 3; c++) d[c] = pos[3 * ib + c] - pos[3 * ia + c];
    or_min_image(s, d);
    double drr = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    double dr = sqrt(drr);
    double dri = 1.0 / dr;
    double rr = dr - seq[i];
    double fr = -k[i] * rr * 2.0;
    eurey += -(fr * rr * 0.5);
    for (int c = 0; c < 3; c++) {
      double f = fr * dri * d[c];
      ff[3 * ia + c] -= f;
      ff[3 * ib + c] += f;
    }
  }
  return eurey;
}

/* The dihedral of (a, b, c, d) and the force of a generalised force fr
 * (-dE/dtau) on the four sites, in the operation order of ctorsion.c:80-246
 * and cimproper.c (the two share it).  Returns tau. */
static double or_dihedral(const or_system *s, const double *pos, int ia, int ib, int ic,
                          int id, double (*fr_of)(double tau, const void *par, double *e),
                          const void *par, double *e, double *ff) {
  double dab[3], dbc[3], dcd[3];
  for (int c = 0; c < 3; c++) {
    dab[c] = pos[3 * ib + c] - pos[3 * ia + c];
    dbc[c] = pos[3 * ic + c] - pos[3 * ib + c];
    dcd[c] = pos[3 * id + c] - pos[3 * ic + c];
  }
  or_min_image(s, dab);
  or_min_image(s, dbc);
  or_min_image(s, dcd);
  double rab = sqrt(dab[0] * dab[0] + dab[1] * dab[1] + dab[2] * dab[2]);
  double irab = 1.0 / rab;
  double eab[3] = {dab[0] * irab, dab[1] * irab, dab[2] * irab};
  double rbc = sqrt(dbc[0] * dbc[0] + dbc[1] * dbc[1] + dbc[2] * dbc[2]);
  double irbc = 1.0 / rbc;
  double ebc[3] = {dbc[0] * irbc, dbc[1] * irbc, dbc[2] * irbc};
  double rcd = sqrt(dcd[0] * dcd[0] + dcd[1] * dcd[1] + dcd[2] * dcd[2]);
  double ircd = 1.0 / rcd;
  double ecd[3] = {dcd[0] * ircd, dcd[1] * ircd, dcd[2] * ircd};
  /* u = eab x ebc, w = ecd x ebc and the bend cosines at b and c */
  double u[3] = {eab[1] * ebc[2] - eab[2] * ebc[1], eab[2] * ebc[0] - eab[0] * ebc[2],
                 eab[0] * ebc[1] - eab[1] * ebc[0]};
  double cosb = -(eab[0] * ebc[0] + eab[1] * ebc[1] + eab[2] * ebc[2]);
  double isinb2 = 1.0 / (1.0 - cosb * cosb);
  double isinb = sqrt(isinb2);
  double w[3] = {ecd[1] * ebc[2] - ecd[2] * ebc[1], ecd[2] * ebc[0] - ecd[0] * ebc[2],
                 ecd[0] * ebc[1] - ecd[1] * ebc[0]};
  double cosc = -(ecd[0] * ebc[0] + ecd[1] * ebc[1] + ecd[2] * ebc[2]);
  double isinc2 = 1.0 / (1.0 - cosc * cosc);
  double isinc = sqrt(isinc2);
  /* sign from (u x w) . ebc, angle from u . w */
  double x0 = -(u[1] * w[2] - u[2] * w[1]);
  double x1 = -(u[2] * w[0] - u[0] * w[2]);
  double x2 = -(u[0] * w[1] - u[1] * w[0]);
  double num = (x0 * ebc[0] + x1 * ebc[1] + x2 * ebc[2]);
  double sgn = num >= 0.0 ? 1.0 : -1.0;
  double costau = -(u[0] * w[0] + u[1] * w[1] + u[2] * w[2]) * isinb * isinc;
  if (costau > 1.0) costau = 1.0;
  if (costau < -1.0) costau = -1.0;
  double tau = sgn * acos(costau);
  double fr = fr_of(tau, par, e);
  double fa = -fr * irab * isinb2;
  double fb1 = fr * (rbc - rab * cosb) * irab * irbc * isinb2;
  double fb2 = fr * cosc * irbc * isinc2;
  double fc1 = fr * (rbc - rcd * cosc) * ircd * irbc * isinc2;
  double fc2 = fr * cosb * irbc * isinb2;
  double fd = -fr * ircd * isinc2;
  for (int c = 0; c < 3; c++) {
    ff[3 * ia + c] += fa * u[c];
    ff[3 * ib + c] += (fb1 * u[c] + fb2 * w[c]);
    ff[3 * ic + c] += fc1 * w[c] + fc2 * u[c];
    ff[3 * id + c] += fd * w[c];
  }
  return tau;
}

typedef struct {
  const double *kphi, *nphi, *delphi; /* 6 each */
} or_tors_par;

/* ctorsion.c:176-188: cosine series, stopping at the first zero kphi */
static double or_tors_fr(double tau, const void *vp, double *e) {
  const or_tors_par *p = (const or_tors_par *)vp;
  double fr = 0.0, et = 0.0;
  for (int t = 0; t < 6; t++) {
    if (p->kphi[t] != 0.0) {
      fr += p->kphi[t] * p->nphi[t] * (sin(p->nphi[t] * tau - p->delphi[t]));
      et += p->kphi[t] * (1 + cos(p->nphi[t] * tau - p->delphi[t]));
    } else {
      break;
    }
  }
  *e = et;
  return fr;
}

double or_ctorsion(const or_system *s, const double *pos, int ntors, const int *abcd,
                   const double *kphi, const double *nphi, const double *delphi, double *ff,
                   double *tau_out) {
  /* ctorsion.c:63-246 */
  double etorsion = 0.0;
  for (int i = 0; i < ntors; i++) {
    or_tors_par p = {kphi + 6 * i, nphi + 6 * i, delphi + 6 * i};
    double et = 0.0;
    double tau = or_dihedral(s, pos, abcd[4 * i], abcd[4 * i + 1], abcd[4 * i + 2],
                             abcd[4 * i + 3], or_tors_fr, &p, &et, ff);
    etorsion += et;
    if (tau_out) tau_out[i] = tau;
  }
  return etorsion;
}

typedef struct {
  double k, eq;
} or_impr_par;

/* cimproper.c: E = kimpr (tau - angeq)^2, fr = -2 kimpr (tau - angeq) */
static double or_impr_fr(double tau, const void *vp, double *e) {
  const or_impr_par *p = (const or_impr_par *)vp;
  double rr = tau - p->eq;
  double fr = -2.0 * p->k * rr;
  *e = -fr * rr * 0.5;
  return fr;
}

double or_cimproper(const or_system *s, const double *pos, int nimpr, const int *abcd,
                    const double *kimpr, const double *angeq, double *ff) {
  /* cimproper.c:55-221 */
  double eimproper = 0.0;
  for (int i = 0; i < nimpr; i++) {
    or_impr_par p = {kimpr[i], angeq[i]};
    double ei = 0.0;
    or_dihedral(s, pos, abcd[4 * i], abcd[4 * i + 1], abcd[4 * i + 2], abcd[4 * i + 3],
                or_impr_fr, &p, &ei, ff);
    eimproper += ei;
  }
  return eimproper;
}

/* ------------------------------------------------------------------------ */
void or_forces(const or_system *s, const double *pos, const int *cnt,
               const int *idx, const int *flag, double sewald, double *ff,
               or_energy *en) {
  /* forces.c:118-219 */
  memset(ff, 0, sizeof(double) * 3 * (size_t)s->n);
  en->bond = or_cbond(s, pos, ff);
  en->bend = or_cbend(s, pos, ff);
  double e5[5], ek[3];
  or_cnonbond_pairs(s, pos, cnt, idx, flag, ff, e5);
  or_pme_calc(s, pos, sewald, ff, ek); /* cnonbond_nblist.c:588 */
  /* cnonbond_nblist.c:601-620 */
  double er0 = e5[2], er1 = e5[2] - e5[3], er2 = e5[4];
  double energy[8];
  energy[0] = e5[0] + er0 - er2 + ek[2];
  energy[1] = energy[0] - e5[1];
  energy[2] = er0 + ek[2] - er2;
  energy[3] = er0 - er1;
  energy[4] = ek[0];
  energy[5] = ek[1];
  energy[6] = er2;
  energy[7] = er0;
  en->nbond = energy[0];
  en->nbonds = energy[1];
  en->coulomb = energy[2];
  en->tewald = energy[2];
  en->rewald = energy[7];
  en->rewalds = energy[3];
  en->kewald = energy[4];
  en->sewald = energy[5];
  en->iewald = energy[6];
}

void or_pbc_all(const or_system *s, double *pos) {
  /* pbc_all.c:23-88 */
  double lx = s->L[0], ly = s->L[1], lz = s->L[2];
  double hx = lx / 2.0, hy = ly / 2.0, hz = lz / 2.0;
  for (int i = 0; i < s->n; i++) {
    double dx = pos[3 * i], dy = pos[3 * i + 1], dz = pos[3 * i + 2];
    double pbcx = 0.0, pbcy = 0.0, pbcz = 0.0;
    while (dx < -hx || dx > hx) {
      if (dx < -hx) pbcx = +lx;
      if (dx > hx) pbcx = -lx;
      dx += pbcx;
    }
    while (dy < -hy || dy > hy) {
      if (dy < -hy) pbcy = +ly;
      if (dy > hy) pbcy = -ly;
      dy += pbcy;
    }
    while (dz < -hz || dz > hz) {
      if (dz < -hz) pbcz = +lz;
      if (dz > hz) pbcz = -lz;
      dz += pbcz;
    }
    pos[3 * i] = dx;
    pos[3 * i + 1] = dy;
    pos[3 * i + 2] = dz;
  }
}

double or_kinet(const or_system *s, const double *vv, const double *uu,
                double *ken_out) {
  /* kinet.c:18-68 */
  double ken[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < s->n; i++) {
    double fac = s->mass[i];
    double vvx = vv[3 * i], vvy = vv[3 * i + 1], vvz = vv[3 * i + 2];
    double uux = uu[3 * i], uuy = uu[3 * i + 1], uuz = uu[3 * i + 2];
    ken[0] += fac * (vvx + uux) * (vvx + uux);
    ken[1] += fac * (vvy + uuy) * (vvx + uux);
    ken[2] += fac * (vvy + uuy) * (vvy + uuy);
    ken[3] += fac * (vvz + uuz) * (vvx + uux);
    ken[4] += fac * (vvz + uuz) * (vvy + uuy);
    ken[5] += fac * (vvz + uuz) * (vvz + uuz);
  }
  for (int i = 0; i < 6; i++) ken[i] *= (0.125) * (NA_ * AU_ * 10.0);
  if (ken_out)
    for (int i = 0; i < 6; i++) ken_out[i] = ken[i];
  return ken[0] + ken[2] + ken[5];
}

void or_integrate_vverlet(const or_system *s, double vscal, double *pos,
                          double *pos_nopbc, double *vv, double *uu,
                          double *ff, const int *cnt, const int *idx,
                          const int *flag, double sewald, or_energy *en) {
  /* integrate_vverlet.c:36-103 */
  double dt = s->dt;
  double dt_h = 0.5 * s->dt;
  for (int i = 0; i < s->n; i++) {
    double imass = 100.0 / s->mass[i];
    for (int c = 0; c < 3; c++)
      vv[3 * i + c] = vscal * (vv[3 * i + c] + dt_h * imass * ff[3 * i + c]);
    for (int c = 0; c < 3; c++) {
      double dd = dt * vv[3 * i + c];
      pos_nopbc[3 * i + c] += dd;
      pos[3 * i + c] += dd;
    }
  }
  or_pbc_all(s, pos);
  or_forces(s, pos, cnt, idx, flag, sewald, ff, en);
  for (int i = 0; i < s->n; i++) {
    double imass = 100.0 / s->mass[i];
    for (int c = 0; c < 3; c++) {
      vv[3 * i + c] = (vv[3 * i + c] + vscal * dt_h * imass * ff[3 * i + c]);
      uu[3 * i + c] = vv[3 * i + c];
    }
  }
}

void or_integrate_nhc(const or_system *s, double time_step, int M, double Q,
                      double nfree, double *zeta, double *vv, double *uu) {
  /* integrate_nhc.c:40-161, Nc = Nys = 1, w[0] = 1 */
#define ZR(j) zeta[3 * (j)]
#define ZV(j) zeta[3 * (j) + 1]
#define ZG(j) zeta[3 * (j) + 2]
  int M1 = M - 1, M2 = M - 2;
  double Nf = nfree;
  double NkT = Nf * KB_ * s->T * 1E-4;
  double kT = KB_ * s->T * 1E-4;
  double kin = or_kinet(s, vv, uu, NULL);
  double akin = 2.0 * kin * 1000.0 * 1E-4 / NA_;
  double scale = 1.0;
  double w0 = 1.0;
  int Nc = 1;
  double dt = time_step * w0 / (double)Nc;
  double dt2 = dt / 2.0, dt4 = dt / 4.0, dt8 = dt / 8.0;
  double AA;
  ZG(0) = (akin - NkT) / Q;
  ZV(M1) += ZG(M1) * dt4;
  for (int j = 0; j < M1; j++) {
    AA = exp(-dt8 * ZV(M1 - j));
    ZV(M2 - j) = ZV(M2 - j) * AA * AA + dt4 * ZG(M2 - j) * AA;
  }
  AA = exp(-dt2 * ZV(0));
  scale = scale * AA;
  for (int j = 0; j < M; j++) ZR(j) += ZV(j) * dt2;
  ZG(0) = (scale * scale * akin - NkT) / Q;
  for (int j = 0; j < M - 1; j++) {
    AA = exp(-dt8 * ZV(j + 1));
    ZV(j) = ZV(j) * AA * AA + dt4 * ZG(j) * AA;
    ZG(j + 1) = (Q * ZV(j) * ZV(j) - kT) / Q;
  }
  ZV(M - 1) += ZG(M - 1) * dt4;
  for (int i = 0; i < 3 * s->n; i++) {
    vv[i] = vv[i] * scale;
    uu[i] = uu[i] * scale;
  }
#undef ZR
#undef ZV
#undef ZG
}

static void en_rec(const or_energy *e, double kin, double *r) {
  r[0] = kin; r[1] = e->bond; r[2] = e->bend; r[3] = e->nbond;
  r[4] = e->nbonds; r[5] = e->coulomb; r[6] = e->rewald; r[7] = e->rewalds;
  r[8] = e->kewald; r[9] = e->sewald; r[10] = e->iewald; r[11] = e->tewald;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int or_run_md(const or_system *s, int nsteps, int nlist_freq, int use_nhc,
              int nhc_M, double nhc_Q, double *pos, double *pos_nopbc,
              double *vv, double *ff, double *zeta, double *rec) {
  return or_run_md_timed(s, nsteps, nlist_freq, use_nhc, nhc_M, nhc_Q, pos, pos_nopbc, vv, ff,
                         zeta, rec, NULL);
}

/* or_run_md with tstamp[i] = monotonic time (s) at the end of step i
 * (tstamp[0]: after the initial list and forces); tstamp may be NULL */
int or_run_md_timed(const or_system *s, int nsteps, int nlist_freq, int use_nhc,
                    int nhc_M, double nhc_Q, double *pos, double *pos_nopbc,
                    double *vv, double *ff, double *zeta, double *rec, double *tstamp) {
  int n = s->n;
  int64_t cap = (int64_t)n * 2000 + 16;
  if (cap > (int64_t)n * n / 2 + 16) cap = (int64_t)n * n / 2 + 16;
  int *cnt = (int *)malloc(sizeof(int) * (size_t)n);
  int *idx = (int *)malloc(sizeof(int) * (size_t)cap);
  int *flag = (int *)malloc(sizeof(int) * (size_t)cap);
  double *uu = (double *)malloc(sizeof(double) * 3 * (size_t)n);
  memcpy(uu, vv, sizeof(double) * 3 * (size_t)n);
  double sewald = or_ewald_self(s);
  double nfree = 3.0 * n - 3.0;
  or_energy en;
  /* main.c:475-496 */
  if (or_nblist(s, pos, cnt, idx, flag, cap, NULL, NULL, NULL, 0) < 0) goto fail;
  or_forces(s, pos, cnt, idx, flag, sewald, ff, &en);
  en_rec(&en, or_kinet(s, vv, uu, NULL), rec);
  if (tstamp) tstamp[0] = now_s();
  for (int i = 1; i <= nsteps; i++) {
    if (i % nlist_freq == 0)
      if (or_nblist(s, pos, cnt, idx, flag, cap, NULL, NULL, NULL, 0) < 0) goto fail;
    if (use_nhc) or_integrate_nhc(s, s->dt, nhc_M, nhc_Q, nfree, zeta, vv, uu);
    or_integrate_vverlet(s, 1.0, pos, pos_nopbc, vv, uu, ff, cnt, idx, flag,
                         sewald, &en);
    if (use_nhc) or_integrate_nhc(s, s->dt, nhc_M, nhc_Q, nfree, zeta, vv, uu);
    en_rec(&en, or_kinet(s, vv, uu, NULL), rec + 12 * i);
    if (tstamp) tstamp[i] = now_s();
  }
  free(cnt); free(idx); free(flag); free(uu);
  return 0;
fail:
  free(cnt); free(idx); free(flag); free(uu);
  return -1;
}

/* ------------------------------------------------------------------------ */
/* classic-Ewald MC energy path                                              */

int or_ewald_nk(int kmax_x, int kmax_y, int kmax_z, int max_k_square) {
  /* ewald.c:104-118 enumeration */
  int t = 0;
  for (int kx = 0; kx <= kmax_x; ++kx)
    for (int ky = -kmax_y; ky <= kmax_y; ++ky)
      for (int kz = -kmax_z; kz <= kmax_z; ++kz) {
        int ksq = kx * kx + ky * ky + kz * kz;
        if (ksq <= max_k_square && ksq != 0) t++;
      }
  return t;
}

static int build_kvec(const or_system *s, int kmax, int mks, double *kvec,
                      int *kv) {
  /* ewald.c:95-118 */
  double kappa = s->kappa;
  double two_pi = 2.0 * PI_;
  double lx = s->L[0], ly = s->L[1], lz = s->L[2];
  double boxv = lx * ly * lz;
  double b = 0.25 / (kappa * kappa);
  int t = 0;
  for (int kx = 0; kx <= kmax; ++kx) {
    double rkx = two_pi * (double)kx / lx;
    for (int ky = -kmax; ky <= kmax; ++ky) {
      double rky = two_pi * (double)ky / ly;
      for (int kz = -kmax; kz <= kmax; ++kz) {
        double rkz = two_pi * (double)kz / lz;
        int ksq = kx * kx + ky * ky + kz * kz;
        if (ksq <= mks && ksq != 0) {
          double rksq = rkx * rkx + rky * rky + rkz * rkz;
          kvec[t] = two_pi * exp(-b * rksq) / rksq / boxv;
          if (kv) {
            kv[3 * t] = kx;
            kv[3 * t + 1] = ky;
            kv[3 * t + 2] = kz;
          }
          ++t;
        }
      }
    }
  }
  return t;
}

typedef struct { double r, i; } cplx;
static cplx cmul(cplx a, cplx b) {
  /* cplx.c C_mul */
  cplx r;
  r.r = a.r * b.r - a.i * b.i;
  r.i = a.r * b.i + b.r * a.i;
  return r;
}
static cplx cconj(cplx a) { a.i = -a.i; return a; }

double or_ewald_kspace_energy(const or_system *s, const double *pos, int kmax,
                              int mks) {
  /* ewald_mc.c:42-324 (energy part, no PRESSURE) */
  int ns = s->n;
  int nk = or_ewald_nk(kmax, kmax, kmax, mks);
  double *kvec = (double *)malloc(sizeof(double) * (size_t)(nk + 1));
  build_kvec(s, kmax, mks, kvec, NULL);
  double two_pi = 2.0 * PI_;
  double iblx = 1.0 / s->L[0], ibly = 1.0 / s->L[1], iblz = 1.0 / s->L[2];
  double tpx = two_pi * iblx, tpy = two_pi * ibly, tpz = two_pi * iblz;
  int KX = kmax + 1, KY = 2 * kmax + 1;
  cplx *ex = (cplx *)malloc(sizeof(cplx) * (size_t)ns * KX);
  cplx *ey = (cplx *)malloc(sizeof(cplx) * (size_t)ns * KY);
  cplx *ez = (cplx *)malloc(sizeof(cplx) * (size_t)ns * KY);
#define EX(i, k) ex[(size_t)(i) * KX + (k)]
#define EY(i, k) ey[(size_t)(i) * KY + (k) + kmax]
#define EZ(i, k) ez[(size_t)(i) * KY + (k) + kmax]
  for (int i = 0; i < ns; i++) {
    double dx = pos[3 * i], dy = pos[3 * i + 1], dz = pos[3 * i + 2];
    EX(i, 0).r = 1.0; EX(i, 0).i = 0.0;
    EY(i, 0).r = 1.0; EY(i, 0).i = 0.0;
    EZ(i, 0).r = 1.0; EZ(i, 0).i = 0.0;
    EX(i, 1).r = cos(tpx * dx); EX(i, 1).i = sin(tpx * dx);
    EY(i, 1).r = cos(tpy * dy); EY(i, 1).i = sin(tpy * dy);
    EZ(i, 1).r = cos(tpz * dz); EZ(i, 1).i = sin(tpz * dz);
    EY(i, -1) = cconj(EY(i, 1));
    EZ(i, -1) = cconj(EZ(i, 1));
  }
  for (int i = 0; i < ns; i++) {
    for (int kx = 2; kx <= kmax; kx++) EX(i, kx) = cmul(EX(i, kx - 1), EX(i, 1));
    for (int ky = 2; ky <= kmax; ky++) {
      EY(i, ky) = cmul(EY(i, ky - 1), EY(i, 1));
      EY(i, -ky) = cconj(EY(i, ky));
    }
    for (int kz = 2; kz <= kmax; kz++) {
      EZ(i, kz) = cmul(EZ(i, kz - 1), EZ(i, 1));
      EZ(i, -kz) = cconj(EZ(i, kz));
    }
  }
  double vk = 0.0;
  int totk = 0;
  for (int ky = -kmax; ky <= kmax; ky++)
    for (int kz = -kmax; kz <= kmax; kz++) {
      int ksq = ky * ky + kz * kz;
      if (ksq <= mks && ksq != 0) {
        double sr = 0.0, si = 0.0;
        for (int i = 0; i < ns; i++) {
          cplx e = cmul(EX(i, 0), cmul(EY(i, ky), EZ(i, kz)));
          sr = sr + s->q[i] * e.r;
          si = si + s->q[i] * e.i;
        }
        vk += kvec[totk] * (sr * sr + si * si);
        totk++;
      }
    }
  for (int kx = 1; kx <= kmax; kx++)
    for (int ky = -kmax; ky <= kmax; ky++)
      for (int kz = -kmax; kz <= kmax; kz++) {
        int ksq = kx * kx + ky * ky + kz * kz;
        if (ksq <= mks) {
          double sr = 0.0, si = 0.0;
          for (int i = 0; i < ns; i++) {
            cplx e = cmul(EX(i, kx), cmul(EY(i, ky), EZ(i, kz)));
            sr = sr + s->q[i] * e.r;
            si = si + s->q[i] * e.i;
          }
          vk += 2.0 * kvec[totk] * (sr * sr + si * si);
          totk++;
        }
      }
#undef EX
#undef EY
#undef EZ
  free(ex); free(ey); free(ez); free(kvec);
  double fconv = (ELEC_ * ELEQ_ * ELEQ_ * NA_ * 0.001);
  return vk * fconv;
}

/* one pair's MC energy terms (enbnd_mc.c / ewald_mc.c:390-606 restated with
 * the reference's minimum image of cnonbond_nblist.c:167-172); with
 * r_switch > 0 the LJ term is switched as in or_cnonbond_pairs (no shift) */
static void mc_pair(const or_system *s, const xtab *t, int a, int b,
                    const double *pa, const double *pb, double rc_ew,
                    double e4[4]) {
  double lx = s->L[0], ly = s->L[1], lz = s->L[2];
  double hx = lx / 2.0, hy = ly / 2.0, hz = lz / 2.0;
  double dx = pa[0] - pb[0], dy = pa[1] - pb[1], dz = pa[2] - pb[2];
  if (dx > hx) dx -= lx;
  else if (dx < -hx) dx += lx;
  if (dy > hy) dy -= ly;
  else if (dy < -hy) dy += ly;
  if (dz > hz) dz -= lz;
  else if (dz < -hz) dz += lz;
  double dr2 = dx * dx + dy * dy + dz * dz;
  int xflag = s->nexcl ? xtab_flag(t, a, b) : 0;
  double rc2 = s->rc * s->rc;
  int nt = s->ntypes;
  if (dr2 <= rc2) {
    double sig = s->lj_sig[s->type[a] * nt + s->type[b]];
    double eps = s->lj_eps[s->type[a] * nt + s->type[b]];
    if (xflag && xflag != 4) { sig = 0.0; eps = 0.0; }
    if ((eps * sig) != 0.0) {
      double sr2 = (sig * sig) / dr2;
      double sr6 = sr2 * sr2 * sr2;
      double sr12 = sr6 * sr6;
      if (s->r_switch > 0.0) {
        /* the CHARMM switch of or_cnonbond_pairs instead of the shift */
        double ron2 = s->r_switch * s->r_switch, elj = eps * (sr12 - 2.0 * sr6);
        if (dr2 > ron2) {
          double c = rc2 - dr2, den = (rc2 - ron2) * (rc2 - ron2) * (rc2 - ron2);
          elj *= c * c * (rc2 + 2.0 * dr2 - 3.0 * ron2) / den;
        }
        e4[0] += elj;
      } else {
        double sr2s = (sig * sig) / rc2;
        double sr6s = sr2s * sr2s * sr2s;
        double sr12s = sr6s * sr6s;
        e4[0] += eps * (sr12 - 2.0 * sr6) - eps * (sr12s - 2.0 * sr6s);
      }
    }
  }
  double rce2 = rc_ew * rc_ew;
  if (dr2 > rce2) return;
  double kappa = s->kappa;
  double fconv = (ELEC_ * ELEQ_ * ELEQ_ * NA_ * 0.001);
  double qqab = s->q[a] * s->q[b] * fconv;
  double qq = qqab;
  if (xflag) qq = (xflag == 4) ? E14FAC_ * qqab : 0.0;
  double dr = sqrt(dr2);
  double dri = 1.0 / dr;
  double erfckr = ref_erfc(kappa * dr);
  if (qq != 0.0) {
    e4[1] += qq * erfckr * dri;
    e4[2] += qq * ref_erfc(kappa * rc_ew) / rc_ew;
  }
  if (xflag) {
    double qq12 = qqab;
    if (xflag == 4) qq12 *= (1.0 - E14FAC_);
    e4[3] += qq12 * (1.0 - erfckr) * dri;
  }
}

void or_mc_pair_energy(const or_system *s, const double *pos, const int *cnt,
                       const int *idx, const int *flag, double rc_ew, int lb,
                       int ub, double e4[4]) {
  (void)flag;
  (void)lb;
  xtab t;
  xtab_build(s, &t);
  e4[0] = e4[1] = e4[2] = e4[3] = 0.0;
  int64_t off = 0;
  for (int a = 0; a < ub && a < s->n; a++) {
    for (int bb = 0; bb < cnt[a]; bb++) {
      int b = idx[off + bb];
      mc_pair(s, &t, a, b, pos + 3 * a, pos + 3 * b, rc_ew, e4);
    }
    off += cnt[a];
  }
  xtab_free(&t);
}

double or_mc_delta_energy(const or_system *s, const double *pos,
                          const double *pos_new, int lb, int ub, int kmax,
                          int mks, double rc_ew, double parts[3]) {
  xtab t;
  xtab_build(s, &t);
  double eo[4] = {0, 0, 0, 0}, en4[4] = {0, 0, 0, 0};
  for (int a = lb; a < ub; a++) {
    for (int b = 0; b < s->n; b++) {
      if (b == a) continue;
      if (b >= lb && b < ub && b < a) continue; /* count moved pairs once */
      mc_pair(s, &t, a, b, pos + 3 * a, pos + 3 * b, rc_ew, eo);
      const double *pb = (b >= lb && b < ub) ? pos_new + 3 * b : pos + 3 * b;
      mc_pair(s, &t, a, b, pos_new + 3 * a, pb, rc_ew, en4);
    }
  }
  xtab_free(&t);
  /* full configuration with the moved atoms replaced */
  double *pn = (double *)malloc(sizeof(double) * 3 * (size_t)s->n);
  memcpy(pn, pos, sizeof(double) * 3 * (size_t)s->n);
  for (int a = lb; a < ub; a++)
    for (int c = 0; c < 3; c++) pn[3 * a + c] = pos_new[3 * a + c];
  double dk = or_ewald_kspace_energy(s, pn, kmax, mks) -
              or_ewald_kspace_energy(s, pos, kmax, mks);
  free(pn);
  double dreal = (en4[1] - eo[1]) - (en4[3] - eo[3]);
  double dlj = en4[0] - eo[0];
  if (parts) {
    parts[0] = dk;
    parts[1] = dreal;
    parts[2] = dlj;
  }
  return dk + dreal + dlj;
}

/* ---- counter-based random numbers and replica exchange ---- */

void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  /* Salmon et al., SC'11: ten rounds; multipliers 0xD2511F53 / 0xCD9E8D57,
   * key increments 0x9E3779B9 / 0xBB67AE85 between rounds */
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

double or_uniform(uint64_t seed, uint32_t tag, uint64_t event, uint32_t lane) {
  uint32_t c[4] = {lane, (uint32_t)event, (uint32_t)(event >> 32), tag};
  uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  or_philox4x32_10(c, k, o);
  uint64_t w = ((uint64_t)o[0] << 32) | o[1];
  return (double)(w >> 11) * (1.0 / 9007199254740992.0);
}

#define OR_TAG_EXCHANGE 0x52455831u

int or_rex_attempt(int R, const double *T_slot, const double *potens_box, int *slot_box,
                   uint64_t attempt, uint64_t seed, int *vmode, double *vfac) {
  /* swap_box.c:5-86 on temperature slots; pairs alternate as repexch.c:273-301 */
  int nacc = 0;
  for (int r = 0; r < R; r++) vmode[r] = 0;
  for (int s = (int)(attempt & 1u); s + 1 < R; s += 2) {
    int r1 = slot_box[s], r2 = slot_box[s + 1];
    double kT1 = ((KB_ * NA_) * T_slot[s]) * .001;      /* read_sim.c:351 */
    double kT2 = ((KB_ * NA_) * T_slot[s + 1]) * .001;
    double delta_beta = 1.0 / kT1 - 1.0 / kT2;
    double delta_energy = potens_box[r1] - potens_box[r2];
    double accep_crit = exp(delta_beta * delta_energy);
    if (accep_crit > or_uniform(seed, OR_TAG_EXCHANGE, attempt, (uint32_t)s)) {
      slot_box[s] = r2;
      slot_box[s + 1] = r1;
      double v_scale_1 = sqrt(T_slot[s] / T_slot[s + 1]);
      vmode[r2] = 1; vfac[r2] = v_scale_1;
      vmode[r1] = 2; vfac[r1] = v_scale_1;
      nacc++;
    }
  }
  return nacc;
}

/* ---- Go-model chains (BAOAB Langevin) ---- */

double or_go_forces(int N, const double *pos, int gbase, const int *nat_start, const int *nat_j,
                    const double *nat_r0, const or_go_params *p, double *f) {
  /* pair loop of cnbnd_golik (cgolik.c:644-948) with the chain workload's
   * energy function: natives eps[5(r0/r)^12 - 6(r0/r)^10], others
   * eps (sigma/r)^12 shifted at rc, bonds k (r - r0)^2 */
  double e = 0.0;
  double sr = p->sigma_rep / p->rc_rep, sr6 = sr * sr * sr * sr * sr * sr;
  double shift = p->eps * sr6 * sr6, rc2 = p->rc_rep * p->rc_rep, s2r = p->sigma_rep * p->sigma_rep;
  for (int i = 0; i < 3 * N; i++) f[i] = 0.0;
  for (int i = 0; i < N; i++) {
    const int gi = gbase + i;
    for (int j = i + 1; j < N; j++) {
      if (j - i < p->min_sep) continue;
      int native = 0;
      double r02 = 0.0;
      for (int q = nat_start[gi]; q < nat_start[gi + 1]; q++)
        if (nat_j[q] == gbase + j) { native = 1; r02 = nat_r0[q] * nat_r0[q]; }
      double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1],
             dz = pos[3 * i + 2] - pos[3 * j + 2];
      double r2 = dx * dx + dy * dy + dz * dz, fs;
      if (native) {
        double s2 = r02 / r2, s10 = s2 * s2 * s2 * s2 * s2, s12 = s10 * s2;
        e += p->eps * (5.0 * s12 - 6.0 * s10);
        fs = 60.0 * p->eps * (s12 - s10) / r2;
      } else {
        if (r2 >= rc2) continue;
        double s2 = s2r / r2, s6 = s2 * s2 * s2, s12 = s6 * s6;
        e += p->eps * s12 - shift;
        fs = 12.0 * p->eps * s12 / r2;
      }
      f[3 * i] += fs * dx; f[3 * i + 1] += fs * dy; f[3 * i + 2] += fs * dz;
      f[3 * j] -= fs * dx; f[3 * j + 1] -= fs * dy; f[3 * j + 2] -= fs * dz;
    }
  }
  for (int i = 0; i + 1 < N; i++) {  /* cbond.c:104-105 convention */
    double dx = pos[3 * i] - pos[3 * i + 3], dy = pos[3 * i + 1] - pos[3 * i + 4],
           dz = pos[3 * i + 2] - pos[3 * i + 5];
    double r = sqrt(dx * dx + dy * dy + dz * dz), dr = r - p->r_bond;
    e += p->k_bond * dr * dr;
    double fs = -2.0 * p->k_bond * dr / r;
    f[3 * i] += fs * dx; f[3 * i + 1] += fs * dy; f[3 * i + 2] += fs * dz;
    f[3 * i + 3] -= fs * dx; f[3 * i + 4] -= fs * dy; f[3 * i + 5] -= fs * dz;
  }
  return e;
}

#define OR_TAG_GO 0x474F4C31u

static void go_normals(uint64_t seed, uint32_t bead, uint64_t step, double z[3]) {
  uint32_t c[4] = {bead, (uint32_t)step, (uint32_t)(step >> 32), OR_TAG_GO};
  uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  or_philox4x32_10(c, k, o);
  double u1 = (double)((o[0] >> 8) + 1u) * (1.0 / 16777216.0);
  double u2 = (double)(o[1] >> 8) * (1.0 / 16777216.0);
  double u3 = (double)((o[2] >> 8) + 1u) * (1.0 / 16777216.0);
  double u4 = (double)(o[3] >> 8) * (1.0 / 16777216.0);
  double ra = sqrt(-2.0 * log(u1)), rb = sqrt(-2.0 * log(u3));
  z[0] = ra * cos(2.0 * PI_ * u2);
  z[1] = ra * sin(2.0 * PI_ * u2);
  z[2] = rb * cos(2.0 * PI_ * u4);
}

double or_go_baoab(int N, double *pos, double *vel, int gbase, const int *nat_start,
                   const int *nat_j, const double *nat_r0, const or_go_params *p, double T,
                   uint64_t seed, uint64_t step0, int nsteps) {
  /* B A O A B (Leimkuhler & Matthews 2013); a = 100 F / m (A/ps^2), kT as
   * read_sim.c:351, the O step's normals by Box-Muller on Philox draws */
  double *f = (double *)malloc(sizeof(double) * 3 * (size_t)N);
  double e = or_go_forces(N, pos, gbase, nat_start, nat_j, nat_r0, p, f);
  double c1 = exp(-p->gamma * p->dt), c2 = sqrt(1.0 - c1 * c1);
  double kT = ((KB_ * NA_) * T) * .001;
  double sv = sqrt(100.0 / p->mass) * sqrt(kT) * c2;
  double hdt = 0.5 * p->dt, ha = 0.5 * p->dt * (100.0 / p->mass);
  for (int s = 0; s < nsteps; s++) {
    for (int i = 0; i < N; i++) {
      double z[3];
      go_normals(seed, (uint32_t)(gbase + i), step0 + (uint64_t)s, z);
      for (int a = 0; a < 3; a++) {
        double v = vel[3 * i + a] + ha * f[3 * i + a];
        double x = pos[3 * i + a] + hdt * v;
        v = c1 * v + sv * z[a];
        pos[3 * i + a] = x + hdt * v;
        vel[3 * i + a] = v;
      }
    }
    e = or_go_forces(N, pos, gbase, nat_start, nat_j, nat_r0, p, f);
    for (int i = 0; i < 3 * N; i++) vel[i] += ha * f[i];
  }
  free(f);
  return e;
}

/* ---- the reference's own Go model (cgolik.c) ---- */

double or_go_hc_term(int N, const double *pos, int gbase, const int *nat_start, const int *nat_j,
                     const double *nat_r0, const or_go_hc_params *p, const double *bond_r0,
                     const double *bend_t0, int term, double *f, double *e2) {
  const double eps = p->eps;
  double e = 0.0;
  for (int i = 0; i < 3 * N; i++) f[i] = 0.0;
  if (term == 0) {  /* cbb_golik, cgolik.c:56-104 */
    double k1 = -eps;
    double k2 = k1 * 100;
    for (int i = 0; i + 1 < N; i++) {
      int ia = i, ib = i + 1;
      double dx = pos[3 * ib] - pos[3 * ia];
      double dy = pos[3 * ib + 1] - pos[3 * ia + 1];
      double dz = pos[3 * ib + 2] - pos[3 * ia + 2];
      double drr = dx * dx + dy * dy + dz * dz;
      double dr = sqrt(drr);
      double dri = 1.0 / dr;
      double rr = dr - bond_r0[i];
      double rr2 = rr * rr;
      double fr1 = k1 * rr * 2.0;
      double fr2 = k2 * rr * rr2 * 4.0;
      e += -rr * (fr1 * 0.5 + fr2 * 0.25);
      double fr = fr1 + fr2;
      double fx = fr * dri * dx, fy = fr * dri * dy, fz = fr * dri * dz;
      f[3 * ia] -= fx; f[3 * ia + 1] -= fy; f[3 * ia + 2] -= fz;
      f[3 * ib] += fx; f[3 * ib + 1] += fy; f[3 * ib + 2] += fz;
    }
  } else if (term == 1) {  /* cba_golik, cgolik.c:204-296 (k_theta = -10 eps) */
    double k_theta = -10.0 * eps;
    for (int i = 0; i + 2 < N; i++) {
      int ia = i, ib = i + 1, ic = i + 2;
      double dax = pos[3 * ia] - pos[3 * ib], day = pos[3 * ia + 1] - pos[3 * ib + 1],
             daz = pos[3 * ia + 2] - pos[3 * ib + 2];
      double dcx = pos[3 * ic] - pos[3 * ib], dcy = pos[3 * ic + 1] - pos[3 * ib + 1],
             dcz = pos[3 * ic + 2] - pos[3 * ib + 2];
      double drai = 1.0 / sqrt(dax * dax + day * day + daz * daz);
      double erax = dax * drai, eray = day * drai, eraz = daz * drai;
      double drci = 1.0 / sqrt(dcx * dcx + dcy * dcy + dcz * dcz);
      double ercx = dcx * drci, ercy = dcy * drci, ercz = dcz * drci;
      double cosphi = erax * ercx + eray * ercy + eraz * ercz;
      double phi = acos(cosphi);
      double isinphi = 1.0 / sqrt(1.0 - cosphi * cosphi);
      double rr = phi - bend_t0[i];
      double fr = k_theta * rr * 2.0;
      e += -fr * rr * 0.5;
      double irasin = drai * isinphi * fr;
      double ircsin = drci * isinphi * fr;
      double fxa = (erax * cosphi - ercx) * irasin, fya = (eray * cosphi - ercy) * irasin,
             fza = (eraz * cosphi - ercz) * irasin;
      double fxc = (ercx * cosphi - erax) * ircsin, fyc = (ercy * cosphi - eray) * ircsin,
             fzc = (ercz * cosphi - eraz) * ircsin;
      f[3 * ia] += fxa; f[3 * ia + 1] += fya; f[3 * ia + 2] += fza;
      f[3 * ib] += -(fxa + fxc); f[3 * ib + 1] += -(fya + fyc); f[3 * ib + 2] += -(fza + fzc);
      f[3 * ic] += fxc; f[3 * ic + 1] += fyc; f[3 * ic + 2] += fzc;
    }
  } else if (term == 2) {  /* cda_golik, cgolik.c:399-610 (k_phi = 0.2 eps, 3-fold) */
    double k_phi = 0.2 * eps;
    for (int i = 0; i + 3 < N; i++) {
      int ia = i, ib = i + 1, ic = i + 2, id = i + 3;
      double dabx = pos[3 * ib] - pos[3 * ia], daby = pos[3 * ib + 1] - pos[3 * ia + 1],
             dabz = pos[3 * ib + 2] - pos[3 * ia + 2];
      double dbcx = pos[3 * ic] - pos[3 * ib], dbcy = pos[3 * ic + 1] - pos[3 * ib + 1],
             dbcz = pos[3 * ic + 2] - pos[3 * ib + 2];
      double dcdx = pos[3 * id] - pos[3 * ic], dcdy = pos[3 * id + 1] - pos[3 * ic + 1],
             dcdz = pos[3 * id + 2] - pos[3 * ic + 2];
      double rab = sqrt(dabx * dabx + daby * daby + dabz * dabz);
      double irab = 1.0 / rab;
      double erabx = dabx * irab, eraby = daby * irab, erabz = dabz * irab;
      double rbc = sqrt(dbcx * dbcx + dbcy * dbcy + dbcz * dbcz);
      double irbc = 1.0 / rbc;
      double erbcx = dbcx * irbc, erbcy = dbcy * irbc, erbcz = dbcz * irbc;
      double rcd = sqrt(dcdx * dcdx + dcdy * dcdy + dcdz * dcdz);
      double ircd = 1.0 / rcd;
      double ercdx = dcdx * ircd, ercdy = dcdy * ircd, ercdz = dcdz * ircd;
      double abbcx = eraby * erbcz - erabz * erbcy;
      double abbcy = erabz * erbcx - erabx * erbcz;
      double abbcz = erabx * erbcy - eraby * erbcx;
      double cosb = -(erabx * erbcx + eraby * erbcy + erabz * erbcz);
      double isinb2 = 1.0 / (1.0 - cosb * cosb);
      double isinb = sqrt(isinb2);
      double dccbx = ercdy * erbcz - ercdz * erbcy;
      double dccby = ercdz * erbcx - ercdx * erbcz;
      double dccbz = ercdx * erbcy - ercdy * erbcx;
      double cosc = -(ercdx * erbcx + ercdy * erbcy + ercdz * erbcz);
      double isinc2 = 1.0 / (1.0 - cosc * cosc);
      double isinc = sqrt(isinc2);
      double abcdx = -(abbcy * dccbz - abbcz * dccby);
      double abcdy = -(abbcz * dccbx - abbcx * dccbz);
      double abcdz = -(abbcx * dccby - abbcy * dccbx);
      double num = (abcdx * erbcx + abcdy * erbcy + abcdz * erbcz);
      double signum = num >= 0.0 ? 1.0 : -1.0;
      double costau = -(abbcx * dccbx + abbcy * dccby + abbcz * dccbz) * isinb * isinc;
      if (costau > 1.0) costau = 1.0;
      if (costau < -1.0) costau = -1.0;
      double tau = signum * acos(costau);
      double fr = k_phi * 3.0 * (sin(3.0 * tau - 0.0));
      e += k_phi * (1 + cos(3.0 * tau - 0.0));
      double fa = -fr * irab * isinb2;
      f[3 * ia] += fa * abbcx; f[3 * ia + 1] += fa * abbcy; f[3 * ia + 2] += fa * abbcz;
      double fb1 = fr * (rbc - rab * cosb) * irab * irbc * isinb2;
      double fb2 = fr * cosc * irbc * isinc2;
      f[3 * ib] += (fb1 * abbcx + fb2 * dccbx);
      f[3 * ib + 1] += (fb1 * abbcy + fb2 * dccby);
      f[3 * ib + 2] += (fb1 * abbcz + fb2 * dccbz);
      double fc1 = fr * (rbc - rcd * cosc) * ircd * irbc * isinc2;
      double fc2 = fr * cosb * irbc * isinb2;
      f[3 * ic] += fc1 * dccbx + fc2 * abbcx;
      f[3 * ic + 1] += fc1 * dccby + fc2 * abbcy;
      f[3 * ic + 2] += fc1 * dccbz + fc2 * abbcz;
      double fd = -fr * ircd * isinc2;
      f[3 * id] += fd * dccbx; f[3 * id + 1] += fd * dccby; f[3 * id + 2] += fd * dccbz;
    }
  } else {  /* cnbnd_golik, cgolik.c:644-948 (protein sites, no solvent) */
    const double factor = pow(2.0, -(1.0 / 6.0));
    double rc2 = p->rc * p->rc, rc2_rep = p->d_rep * p->d_rep;
    double enonbond = 0.0, enonbonds = 0.0, enonnative = 0.0;
    for (int a = 0; a < N - 1; a++) {
      double fxa = 0.0, fya = 0.0, fza = 0.0;
      double ax = pos[3 * a], ay = pos[3 * a + 1], az = pos[3 * a + 2];
      for (int b = a + 1; b < N; b++) {
        double dx = ax - pos[3 * b], dy = ay - pos[3 * b + 1], dz = az - pos[3 * b + 2];
        double dr2 = dx * dx + dy * dy + dz * dz;
        if (dr2 > rc2) continue;
        int flag = 0;
        double sig = factor * p->d_rep, pe = eps;
        for (int q = nat_start[gbase + a]; q < nat_start[gbase + a + 1]; q++)
          if (nat_j[q] == gbase + b) { flag = 1; sig = factor * nat_r0[q]; }
        if (b == a + 1) { flag = 0; sig = 0.0; pe = 0.0; }  /* read_golik.c:99-110 */
        if (flag == 0 && dr2 > rc2_rep) continue;
        double force = 0.0;
        if ((pe * sig) != 0.0) {
          double sr2 = (sig * sig) / dr2, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
          double sr2s = (sig * sig) / rc2, sr6s = sr2s * sr2s * sr2s, sr12s = sr6s * sr6s;
          force = (48.0 * pe / dr2) * (sr12 - 0.5 * sr6);
          double enbnd = 4.0 * pe * (sr12 - sr6);
          double enbnds = 4.0 * pe * (sr12s - sr6s);
          if (flag == 0) {
            enonnative += (enbnd + pe);
          } else {
            enonbond += enbnd;
            enonbonds += enbnds;
          }
        }
        if (force != 0.0) {
          double fx = force * dx, fy = force * dy, fz = force * dz;
          fxa += fx; fya += fy; fza += fz;
          f[3 * b] -= fx; f[3 * b + 1] -= fy; f[3 * b + 2] -= fz;
        }
      }
      f[3 * a] += fxa; f[3 * a + 1] += fya; f[3 * a + 2] += fza;
    }
    if (e2) {
      e2[0] = enonbond + enonnative;
      e2[1] = enonbond - enonbonds + enonnative;
    }
    e = enonbond - enonbonds + enonnative;
  }
  return e;
}

static double go_hc_all(int N, const double *pos, int gbase, const int *nat_start,
                        const int *nat_j, const double *nat_r0, const or_go_hc_params *hc,
                        const double *bond_r0, const double *bend_t0, double *f) {
  double *t = (double *)malloc(sizeof(double) * 3 * (size_t)N);
  double e = 0.0;
  for (int i = 0; i < 3 * N; i++) f[i] = 0.0;
  for (int term = 0; term < 4; term++) {
    e += or_go_hc_term(N, pos, gbase, nat_start, nat_j, nat_r0, hc, bond_r0, bend_t0, term, t,
                       NULL);
    for (int i = 0; i < 3 * N; i++) f[i] += t[i];
  }
  free(t);
  return e;
}

double or_go_baoab_hc(int N, double *pos, double *vel, int gbase, const int *nat_start,
                      const int *nat_j, const double *nat_r0, const or_go_params *p,
                      const or_go_hc_params *hc, const double *bond_r0, const double *bend_t0,
                      double T, uint64_t seed, uint64_t step0, int nsteps) {
  /* the B A O A B sequence of or_go_baoab with these forces */
  double *f = (double *)malloc(sizeof(double) * 3 * (size_t)N);
  double e = go_hc_all(N, pos, gbase, nat_start, nat_j, nat_r0, hc, bond_r0, bend_t0, f);
  double c1 = exp(-p->gamma * p->dt), c2 = sqrt(1.0 - c1 * c1);
  double kT = ((KB_ * NA_) * T) * .001;
  double sv = sqrt(100.0 / p->mass) * sqrt(kT) * c2;
  double hdt = 0.5 * p->dt, ha = 0.5 * p->dt * (100.0 / p->mass);
  for (int s = 0; s < nsteps; s++) {
    for (int i = 0; i < N; i++) {
      double z[3];
      go_normals(seed, (uint32_t)(gbase + i), step0 + (uint64_t)s, z);
      for (int a = 0; a < 3; a++) {
        double v = vel[3 * i + a] + ha * f[3 * i + a];
        double x = pos[3 * i + a] + hdt * v;
        v = c1 * v + sv * z[a];
        pos[3 * i + a] = x + hdt * v;
        vel[3 * i + a] = v;
      }
    }
    e = go_hc_all(N, pos, gbase, nat_start, nat_j, nat_r0, hc, bond_r0, bend_t0, f);
    for (int i = 0; i < 3 * N; i++) vel[i] += ha * f[i];
  }
  free(f);
  return e;
}
