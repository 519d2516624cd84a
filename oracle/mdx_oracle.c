/*
 * mdx_oracle.c -- CPU restatement of MDynaMix v5.3's force path and
 * integrators, used as the parity oracle for the GPU library.
 *
 * TEST INFRASTRUCTURE ONLY: tests, the smoke check and the benchmark's
 * CPU-baseline leg call it; the product never does.
 *
 * Pinned to the reference's own example run (sample/4nacl.in, its restart
 * file sample/NaCl.dmp and its output sample/4nacl.out, committed as
 * fixtures under tests/golden/): the setup numbers the output prints (box
 * from the density, INIFUR's k-vector count, degrees of freedom, LJ tail
 * corrections per molecule-type pair) agree to the printed digits, and a
 * continuation of that run from its restart file reproduces its averages
 * within stated bars.  The reference binary itself cannot run here
 * (Fortran; no compiler on either machine), so no bit-for-bit comparison
 * with it exists.  Invariants in the tests pin the rest: momentum
 * conservation of pair and bonded forces, finite-difference forces, alpha
 * independence of the Ewald total, NVE energy conservation.
 *
 * Each routine follows the Fortran statement by statement, in double
 * precision, with the same operation order.  Arrays are indexed 1..N as in
 * the Fortran (element 0 unused).  Build flags keep IEEE semantics
 * (-O2 -ffp-contract=off, no fast-math) so that x86 and Arm agree.
 *
 *   ox_chcnb      CHCNB     forces.f:1813-2205
 *   localf        LOCALF    forces.f:813-998
 *   forces_long   FORCES    forces.f:1014-1202
 *   furir         FURIR     forces.f:1217-1339
 *   ox_inifur     INIFUR    forces.f:1356-1449
 *   eterms        ETERMS    forces.f:1482-1676
 *   getbnd        GETBND    forces.f:113-204
 *   getang        GETANG    forces.f:216-309
 *   gettrs        GETTRS    forces.f:323-513
 *   strbnd        STRBND    forces.f:530-800
 *   ox_fforces    FFORCES   forces.f:36-51   (+ CM_ADDF scalar.f:28-60)
 *   ox_slforces   SLFORCES  forces.f:55-73   (+ CM_ADDLF scalar.f:64-84)
 *   ox_allforce   ALLFORCE  forces.f:77-100  (+ CM_ADDLA scalar.f:88-116)
 *   sclfrc        SCLFRC    service.f:182-287
 *   zerofs        ZEROFS    service.f:397-453
 *   ox_getcom     GETCOM    service.f:463-563
 *   ox_getkin     GETKIN    service.f:611-735 (no GETROT)
 *   ox_chkmom     CHKMOM    service.f:1081-1125
 *   reclen        RECLEN    service.f:572-605
 *   getemp        GETEMP    service.f:35-117
 *   pbc           PBC       service.f:953-990
 *   scaling       SCALING   mdstep.f:534-1093
 *   shejk         SHEJK     mdstep.f:1105-1283
 *   ox_double     DOUBLE    mdstep.f:281-530
 *   ox_sultan     SULTAN    mdstep.f:29-260
 *   ox_set_lambda RECINT    mdee.f:86-140
 *   ox_ee_delta   DIFFUR    mdee.f:265-376, DIFEN mdee.f:379-536
 */
#include "mdx_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* common_inc.f:22-33 */
#define A1 0.254829592
#define A2 (-0.284496736)
#define A3 1.421413741
#define A4 (-1.453152027)
#define A5 1.061405429
#define B1 0.3275911
#define PI 3.1415926536
#define TOTPI 1.128379169
#define NT MDX_NTPS

struct ox_state {
  int nstot, nop, ntypes, nsites, nnbt, nrbb, nraa, nrtt, nrbt, nrat, nrrt;
  int nbdmax, nkvm, caps, capl;
  int *itype, *nnum, *nsite, *itm;
  double *massdi, *q;
  double *charge, *mass;
  int *inbt;
  int nspec[NT + 2], nsits[NT + 2], isadr[NT + 2], isaddr[NT + 2],
      iaddr[NT + 2], ipot[NT + 2], nrb[NT + 2], iadb[NT + 2], ishejk[NT + 2],
      iee[NT + 2], lmove[NT + 2];
  double c14el[NT + 2], c14lj[NT + 2], summas[NT + 2];
  double *a6lj, *b12lj, *a6lj0, *b12lj0, *a6_14, *b12_14;
  int mdxt[NT + 2][NT + 2];
  int *nnbb, *inbb;
  int *ib, *jb, *id, *lcon; /* lcon: SHAKE constraint per bond record */
  double *rb, *fb, *db, *ro;
  int *ibi, *jbj, *ibuk;
  double *ra, *fa;
  int *iai, *jaj, *kak, *iauk;
  int *itors, *nmul;
  double *ft, *rt, *ft1, *ft2, *ft3, *ft4, *ft5;
  int *iti, *jtj, *ktk, *ltl, *ituk;
  mdx_params p;
  double boxl, boyl, bozl, hboxl, hboyl, hbozl, boxy3, vol, rssq, short2;
  int lhex, loct;
  double *sx, *sy, *sz, *vx, *vy, *vz, *fx, *fy, *fz, *gx, *gy, *gz, *hx,
      *hy, *hz, *ox, *oy, *oz, *wx, *wy, *wz;
  /* Verlet-skin list mode (not in the reference): squared list radius and
   * the positions of the last list build; list builds counted */
  double rlist2, *rsx, *rsy, *rsz;
  int nbuild;
  /* PULLBACK (forces.f:1756-1799): drag, wells, external field; NSTEP */
  int pull_on, pull_nstep, *pull_atom;
  double *pull_ref;
  mdx_pullback pb;
  double *X, *Y, *Z, *PX, *PY, *PZ;
  int mbsh, mbln;
  int *nbs1, *nbs2, *nbl1, *nbl2;
  int nkv, furir_init;
  double *rkx, *rky, *rkz;
  double boxlo, boylo, bozlo;
  double spei, speei[NT + 2];
  mdx_scalars s;
  double *br, *be, *ar, *ae, *tr, *te;
  mdx_thermo th;
  int lscfl, nthreads;
  char msg[256];
};

#define IDX2(i, j, ld) ((size_t)((i)-1) + (size_t)((j)-1) * (size_t)(ld))

/* Fortran SIGN(A,B): |A| with the sign bit of B, as gfortran on IEEE. */
static double sgn(double a, double b) { return copysign(fabs(a), b); }

static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  return p;
}

static int *copy_i(const int32_t *src, int n) {
  int *d = (int *)xcalloc((size_t)n + 1, sizeof(int));
  if (src)
    for (int i = 0; i < n; ++i) d[i + 1] = src[i];
  return d;
}

static double *copy_d(const double *src, int n) {
  double *d = (double *)xcalloc((size_t)n + 1, sizeof(double));
  if (src)
    for (int i = 0; i < n; ++i) d[i + 1] = src[i];
  return d;
}

/* RECLEN (service.f:572-605): box-dependent quantities. */
static void reclen(ox_state *st, double scx, double scy, double scz) {
  const double cos30 = (double)0.8660254037844386f;
  st->boxl = scx * st->boxl;
  if (st->lhex) {
    st->boyl = st->boxl * cos30;
    st->boxy3 = 0.66666666666666666667 * st->boyl;
    st->bozl = scz * st->bozl;
  } else if (st->loct) {
    st->boxl = (scx + scy + scz) * st->boxl / (3. * scx);
    st->boyl = st->boxl;
    st->bozl = st->boxl;
  } else {
    st->boyl = scy * st->boyl;
    st->bozl = scz * st->bozl;
  }
  st->hboxl = 0.5 * st->boxl;
  st->hboyl = 0.5 * st->boyl;
  st->hbozl = 0.5 * st->bozl;
  st->rssq = st->p.rcut * st->p.rcut;
  st->rlist2 = st->p.rskin > 0. ? (st->p.rcut + st->p.rskin) * (st->p.rcut + st->p.rskin)
                                : st->rssq;
  st->vol = st->boxl * st->boyl * st->bozl;
  if (st->p.icell == 1) st->vol = 0.5 * st->vol;
}

/* Minimum image as inlined in the force loops and PBC (service.f:953-990).
 * hbz is HBOZL everywhere except LOCALF, which tests DZ against HBOXL
 * (forces.f:871); the restatement keeps that. */
static inline void pbc_h(const ox_state *st, double *xx, double *yy,
                         double *zz, double hbz) {
  const double cos30 = (double)0.8660254037844386f;
  const double boxyc = 0.5 / cos30;
  double XX = *xx, YY = *yy, ZZ = *zz;
  if (fabs(XX) > st->hboxl) XX = XX - sgn(st->boxl, XX);
  if (fabs(ZZ) > hbz) ZZ = ZZ - sgn(st->bozl, ZZ);
  if (st->lhex) {
    double XY = boxyc * XX;
    if (YY > st->boxy3 - XY && (XX > 0. || YY > 2. * st->boxy3 - XY)) {
      YY = YY - st->boyl;
      XX = XX - st->hboxl;
      XY = boxyc * XX;
    }
    if (YY < -st->boxy3 - XY && (XX < 0. || YY < -2. * st->boxy3 - XY)) {
      YY = YY + st->boyl;
      XX = XX + st->hboxl;
      XY = boxyc * XX;
    }
    if (YY > st->boxy3 + XY) {
      YY = YY - st->boyl;
      XX = XX + st->hboxl;
      XY = boxyc * XX;
    }
    if (YY < -st->boxy3 + XY) {
      YY = YY + st->boyl;
      XX = XX - st->hboxl;
    }
  } else {
    if (fabs(YY) > st->hboyl) YY = YY - sgn(st->boyl, YY);
  }
  if (st->loct) {
    double corss = st->hboxl *
                   (double)(int)((double)(4.0f / 3.0f) *
                                 (fabs(XX) + fabs(YY) + fabs(ZZ)) / st->boxl);
    XX = XX - sgn(corss, XX);
    YY = YY - sgn(corss, YY);
    ZZ = ZZ - sgn(corss, ZZ);
  }
  *xx = XX;
  *yy = YY;
  *zz = ZZ;
}

static inline void pbc(const ox_state *st, double *x, double *y, double *z) {
  pbc_h(st, x, y, z, st->hbozl);
}

/* ------------------------------------------------------------------ open */
int ox_open(const mdx_dims *d, const mdx_topo *t, const mdx_params *p,
            ox_state **out) {
  ox_state *st = (ox_state *)xcalloc(1, sizeof(ox_state));
  st->nstot = d->nstot;
  st->nop = d->nop;
  st->ntypes = d->ntypes;
  st->nsites = d->nsites;
  st->nnbt = d->nnbt;
  st->nrbb = d->nrbb;
  st->nraa = d->nraa;
  st->nrtt = d->nrtt;
  st->nrbt = d->nrbt;
  st->nrat = d->nrat;
  st->nrrt = d->nrrt;
  st->nbdmax = d->nbdmax;
  st->nkvm = d->nkv_max;
  st->nthreads = 1;
  if (st->ntypes > NT || st->ntypes < 1) {
    free(st);
    return MDX_ERR_ARG;
  }
  int n = st->nstot;
  st->itype = copy_i(t->itype, n);
  st->nnum = copy_i(t->nnum, n);
  st->nsite = copy_i(t->nsite, n);
  st->massdi = copy_d(t->massdi, n);
  st->q = copy_d(t->q, n);
  st->charge = copy_d(t->charge, st->nsites);
  st->mass = copy_d(t->mass, st->nsites);
  st->inbt = copy_i(t->inbt, st->nsites);
  for (int i = 0; i < st->ntypes; ++i) {
    st->nspec[i + 1] = t->nspec[i];
    st->nsits[i + 1] = t->nsits[i];
    st->isadr[i + 1] = t->isadr[i];
    st->isaddr[i + 1] = t->isaddr[i];
    st->iaddr[i + 1] = t->iaddr[i];
    st->ipot[i + 1] = t->ipot[i];
    st->nrb[i + 1] = t->nrb[i];
    st->iadb[i + 1] = t->iadb[i];
    st->ishejk[i + 1] = t->ishejk[i];
    st->iee[i + 1] = t->iee[i];
    st->lmove[i + 1] = t->lmove[i];
    st->c14el[i + 1] = t->c14el[i];
    st->c14lj[i + 1] = t->c14lj[i];
    st->summas[i + 1] = t->summas[i];
  }
  st->isadr[st->ntypes + 1] = st->isadr[st->ntypes] + st->nsits[st->ntypes];
  st->isaddr[st->ntypes + 1] =
      st->isaddr[st->ntypes] + st->nsits[st->ntypes] * st->nspec[st->ntypes];
  st->iaddr[st->ntypes + 1] = st->iaddr[st->ntypes] + st->nspec[st->ntypes];
  int nb = st->nnbt;
  double **tabs[6] = {&st->a6lj, &st->b12lj, &st->a6lj0,
                      &st->b12lj0, &st->a6_14, &st->b12_14};
  const double *srcs[6] = {t->a6lj, t->b12lj, t->a6lj0,
                           t->b12lj0, t->a6_14, t->b12_14};
  for (int k = 0; k < 6; ++k) {
    double *a = (double *)xcalloc((size_t)nb * nb, sizeof(double));
    for (int j = 1; j <= nb; ++j)
      for (int i = 1; i <= nb; ++i)
        a[IDX2(i, j, nb)] = srcs[k][IDX2(i, j, t->ld_lj)];
    *tabs[k] = a;
  }
  for (int j = 1; j <= st->ntypes; ++j)
    for (int i = 1; i <= st->ntypes; ++i)
      st->mdxt[i][j] = t->mdx[IDX2(i, j, t->ld_mdx)];
  st->nnbb = copy_i(t->nnbb, n);
  st->inbb = (int *)xcalloc((size_t)n * (st->nbdmax > 0 ? st->nbdmax : 1),
                            sizeof(int));
  for (int k = 1; k <= st->nbdmax; ++k)
    for (int i = 1; i <= n; ++i)
      st->inbb[IDX2(i, k, n)] = t->inbb[IDX2(i, k, t->ld_inbb)];
  st->ib = copy_i(t->ib, st->nrbb);
  st->jb = copy_i(t->jb, st->nrbb);
  st->id = copy_i(t->id, st->nrbb);
  st->lcon = (int *)xcalloc((size_t)st->nrbb + 1, sizeof(int));
  for (int m = 1; m <= st->nrbb; ++m) st->lcon[m] = t->lcon ? t->lcon[m - 1] : st->id[m] != 2;
  st->rb = copy_d(t->rb, st->nrbb);
  st->fb = copy_d(t->fb, st->nrbb);
  st->db = copy_d(t->db, st->nrbb);
  st->ro = copy_d(t->ro, st->nrbb);
  st->ibi = copy_i(t->ibi, st->nrbt);
  st->jbj = copy_i(t->jbj, st->nrbt);
  st->ibuk = copy_i(t->ibuk, st->nrbt);
  st->ra = copy_d(t->ra, st->nraa);
  st->fa = copy_d(t->fa, st->nraa);
  st->iai = copy_i(t->iai, st->nrat);
  st->jaj = copy_i(t->jaj, st->nrat);
  st->kak = copy_i(t->kak, st->nrat);
  st->iauk = copy_i(t->iauk, st->nrat);
  st->itors = copy_i(t->itors, st->nrtt);
  st->nmul = copy_i(t->nmul, st->nrtt);
  st->ft = copy_d(t->ft, st->nrtt);
  st->rt = copy_d(t->rt, st->nrtt);
  st->ft1 = copy_d(t->ft1, st->nrtt);
  st->ft2 = copy_d(t->ft2, st->nrtt);
  st->ft3 = copy_d(t->ft3, st->nrtt);
  st->ft4 = copy_d(t->ft4, st->nrtt);
  st->ft5 = copy_d(t->ft5, st->nrtt);
  st->iti = copy_i(t->iti, st->nrrt);
  st->jtj = copy_i(t->jtj, st->nrrt);
  st->ktk = copy_i(t->ktk, st->nrrt);
  st->ltl = copy_i(t->ltl, st->nrrt);
  st->ituk = copy_i(t->ituk, st->nrrt);
  st->itm = (int *)xcalloc((size_t)st->nop + 1, sizeof(int));
  for (int i = 1; i <= n; ++i) st->itm[st->nnum[i]] = st->itype[i];
  double **arr[] = {&st->sx, &st->sy, &st->sz, &st->vx, &st->vy, &st->vz,
                    &st->fx, &st->fy, &st->fz, &st->gx, &st->gy, &st->gz,
                    &st->hx, &st->hy, &st->hz, &st->ox, &st->oy, &st->oz,
                    &st->wx, &st->wy, &st->wz, &st->rsx, &st->rsy, &st->rsz};
  for (size_t k = 0; k < sizeof(arr) / sizeof(arr[0]); ++k)
    *arr[k] = (double *)xcalloc((size_t)n + 1, sizeof(double));
  double **marr[] = {&st->X, &st->Y, &st->Z, &st->PX, &st->PY, &st->PZ};
  for (int k = 0; k < 6; ++k)
    *marr[k] = (double *)xcalloc((size_t)st->nop + 1, sizeof(double));
  st->caps = d->cap_short > 0 ? d->cap_short : 64;
  st->capl = d->cap_long > 0 ? d->cap_long : 1000;
  st->nbs1 = (int *)xcalloc((size_t)st->caps * n + 1, sizeof(int));
  st->nbs2 = (int *)xcalloc((size_t)st->caps * n + 1, sizeof(int));
  st->nbl1 = (int *)xcalloc((size_t)st->capl * n + 1, sizeof(int));
  st->nbl2 = (int *)xcalloc((size_t)st->capl * n + 1, sizeof(int));
  st->rkx = (double *)xcalloc((size_t)st->nkvm + 1, sizeof(double));
  st->rky = (double *)xcalloc((size_t)st->nkvm + 1, sizeof(double));
  st->rkz = (double *)xcalloc((size_t)st->nkvm + 1, sizeof(double));
  st->br = (double *)xcalloc((size_t)st->nrbb + 1, sizeof(double));
  st->be = (double *)xcalloc((size_t)st->nrbb + 1, sizeof(double));
  st->ar = (double *)xcalloc((size_t)st->nraa + 1, sizeof(double));
  st->ae = (double *)xcalloc((size_t)st->nraa + 1, sizeof(double));
  st->tr = (double *)xcalloc((size_t)st->nrtt + 1, sizeof(double));
  st->te = (double *)xcalloc((size_t)st->nrtt + 1, sizeof(double));
  ox_set_params(st, p);
  *out = st;
  return MDX_OK;
}

int ox_set_params(ox_state *st, const mdx_params *p) {
  st->p = *p;
  st->lhex = p->icell == 2;
  st->loct = p->icell == 1;
  st->boxl = p->boxl;
  st->boyl = p->boyl;
  st->bozl = p->bozl;
  st->th.boxl = p->boxl;
  st->th.boyl = p->boyl;
  st->th.bozl = p->bozl;
  if (st->lhex) st->boxy3 = 0.66666666666666666667 * st->boyl;
  reclen(st, 1.0, 1.0, 1.0);
  st->short2 = p->rshort * p->rshort;
  st->furir_init = 0;
  return MDX_OK;
}

void ox_close(ox_state *st) {
  if (!st) return;
  void *ptrs[] = {st->itype, st->nnum, st->nsite, st->itm, st->massdi, st->q,
                  st->charge, st->mass, st->inbt, st->a6lj, st->b12lj,
                  st->a6lj0, st->b12lj0, st->a6_14, st->b12_14, st->nnbb,
                  st->inbb, st->ib, st->jb, st->id, st->lcon, st->rb, st->fb, st->db,
                  st->ro, st->ibi, st->jbj, st->ibuk, st->ra, st->fa, st->iai,
                  st->jaj, st->kak, st->iauk, st->itors, st->nmul, st->ft,
                  st->rt, st->ft1, st->ft2, st->ft3, st->ft4, st->ft5, st->iti,
                  st->jtj, st->ktk, st->ltl, st->ituk, st->sx, st->sy, st->sz,
                  st->vx, st->vy, st->vz, st->fx, st->fy, st->fz, st->gx,
                  st->gy, st->gz, st->hx, st->hy, st->hz, st->ox, st->oy,
                  st->oz, st->wx, st->wy, st->wz, st->rsx, st->rsy, st->rsz, st->pull_atom,
                  st->pull_ref, st->X, st->Y, st->Z, st->PX,
                  st->PY, st->PZ, st->nbs1, st->nbs2, st->nbl1, st->nbl2,
                  st->rkx, st->rky, st->rkz, st->br, st->be, st->ar, st->ae,
                  st->tr, st->te};
  for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); ++k) free(ptrs[k]);
  free(st);
}

const char *ox_last_error(const ox_state *st) { return st ? st->msg : ""; }

int ox_set_threads(ox_state *st, int n) {
  st->nthreads = n > 0 ? n : 1;
  return MDX_OK;
}

int ox_set_state(ox_state *st, const double *sx, const double *sy,
                 const double *sz, const double *vx, const double *vy,
                 const double *vz, const mdx_thermo *th) {
  for (int i = 0; i < st->nstot; ++i) {
    st->sx[i + 1] = sx[i];
    st->sy[i + 1] = sy[i];
    st->sz[i + 1] = sz[i];
    st->vx[i + 1] = vx[i];
    st->vy[i + 1] = vy[i];
    st->vz[i + 1] = vz[i];
  }
  st->nbuild = th ? th->list_builds : 0;
  if (th) {
    double bl = st->boxl, by = st->boyl, bz = st->bozl;
    st->th = *th;
    if (th->boxl > 0.0) {
      st->boxl = th->boxl;
      st->boyl = th->boyl;
      st->bozl = th->bozl;
      if (st->lhex) st->boxy3 = 0.66666666666666666667 * st->boyl;
      reclen(st, 1.0, 1.0, 1.0);
    } else {
      st->th.boxl = bl;
      st->th.boyl = by;
      st->th.bozl = bz;
    }
  }
  /* molecular centres as the driver's last GETCOM left them: wrapped COM of
   * the given coordinates, coordinates untouched */
  {
    int N = 0, I = 0;
    for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP)
      for (int J = 1; J <= st->nspec[ITYP]; ++J) {
        I = I + 1;
        double x = 0., y = 0., z = 0.;
        for (int IS = st->isadr[ITYP] + 1; IS <= st->isadr[ITYP + 1]; ++IS) {
          N = N + 1;
          x = x + st->mass[IS] * st->sx[N];
          y = y + st->mass[IS] * st->sy[N];
          z = z + st->mass[IS] * st->sz[N];
        }
        x = x / st->summas[ITYP];
        y = y / st->summas[ITYP];
        z = z / st->summas[ITYP];
        pbc(st, &x, &y, &z);
        st->X[I] = x;
        st->Y[I] = y;
        st->Z[I] = z;
      }
  }
  return MDX_OK;
}

static void sync_thermo_box(ox_state *st) {
  st->th.boxl = st->boxl;
  st->th.boyl = st->boyl;
  st->th.bozl = st->bozl;
  st->th.vol = st->vol;
}

int ox_get_state(ox_state *st, double *sx, double *sy, double *sz, double *vx,
                 double *vy, double *vz, mdx_thermo *th) {
  for (int i = 0; i < st->nstot; ++i) {
    if (sx) sx[i] = st->sx[i + 1];
    if (sy) sy[i] = st->sy[i + 1];
    if (sz) sz[i] = st->sz[i + 1];
    if (vx) vx[i] = st->vx[i + 1];
    if (vy) vy[i] = st->vy[i + 1];
    if (vz) vz[i] = st->vz[i + 1];
  }
  sync_thermo_box(st);
  st->th.list_builds = st->nbuild;
  if (th) *th = st->th;
  return MDX_OK;
}

int ox_get_forces(ox_state *st, int which, double *fx, double *fy,
                  double *fz) {
  const double *ax = which == 1 ? st->hx : which == 2 ? st->gx : st->fx;
  const double *ay = which == 1 ? st->hy : which == 2 ? st->gy : st->fy;
  const double *az = which == 1 ? st->hz : which == 2 ? st->gz : st->fz;
  for (int i = 0; i < st->nstot; ++i) {
    fx[i] = ax[i + 1];
    fy[i] = ay[i + 1];
    fz[i] = az[i + 1];
  }
  return MDX_OK;
}

int ox_get_bonded_averages(ox_state *st, double *br, double *be, double *ar,
                           double *ae, double *tr, double *te) {
  for (int i = 0; i < st->nrbb; ++i) {
    if (br) br[i] = st->br[i + 1];
    if (be) be[i] = st->be[i + 1];
  }
  for (int i = 0; i < st->nraa; ++i) {
    if (ar) ar[i] = st->ar[i + 1];
    if (ae) ae[i] = st->ae[i + 1];
  }
  for (int i = 0; i < st->nrtt; ++i) {
    if (tr) tr[i] = st->tr[i + 1];
    if (te) te[i] = st->te[i + 1];
  }
  return MDX_OK;
}

/* ---------------------------------------------------------------- CHCNB */
/* Classify one candidate pair of the strip loop (forces.f:1838-2134).
 * Returns 0 none, 1 short, 2 long, 3 short 1-4, -1 excluded. */
static inline int chcnb_pair(const ox_state *st, int I, int J, int imol) {
  int jmol = st->nnum[J];
  double DX = st->sx[I] - st->sx[J];
  double DY = st->sy[I] - st->sy[J];
  double DZ = st->sz[I] - st->sz[J];
  pbc(st, &DX, &DY, &DZ);
  double RR2 = DX * DX + DY * DY + DZ * DZ;
  double RRM = RR2; /* Ewald: atomic cutoff */
  if (st->p.lmnbl) {
    /* molecular cutoff: small molecules (at most MMOL = 5 sites) are in or
     * out of the list as a whole, by their centre of mass (forces.f:1882-1936) */
    const int MMOL = 5;
    int NMI = st->nsits[st->itype[I]], NMJ = st->nsits[st->itype[J]];
    if (!(NMI > MMOL && NMJ > MMOL)) {
      if (NMI > MMOL && NMJ <= MMOL) {
        DX = st->sx[I] - st->X[jmol]; DY = st->sy[I] - st->Y[jmol]; DZ = st->sz[I] - st->Z[jmol];
      } else if (NMJ > MMOL) {
        DX = st->X[imol] - st->sx[J]; DY = st->Y[imol] - st->sy[J]; DZ = st->Z[imol] - st->sz[J];
      } else {
        DX = st->X[imol] - st->X[jmol]; DY = st->Y[imol] - st->Y[jmol]; DZ = st->Z[imol] - st->Z[jmol];
      }
      pbc(st, &DX, &DY, &DZ);
      RRM = DX * DX + DY * DY + DZ * DZ;
    }
  }
  if (imol == jmol) {
    if (RR2 <= 64.0) {
      int nb = st->nnbb[I];
      for (int K = 1; K <= nb; ++K) {
        int v = st->inbb[IDX2(I, K, st->nstot)];
        if (v == J) return -1;
        if (v == -J) return 3;
      }
    }
  }
  if (RRM <= st->short2) return 1;
  if (RRM <= st->rlist2) return 2; /* RSSQ in the reference; RCUT+skin in skin mode */
  return 0;
}

/* Skin mode (not in the reference): rebuild once some atom has moved more
 * than half the skin (minimum image) since the last build. */
static int skin_moved(ox_state *st) {
  const double h2 = 0.25 * st->p.rskin * st->p.rskin;
  for (int I = 1; I <= st->nstot; ++I) {
    double DX = st->sx[I] - st->rsx[I], DY = st->sy[I] - st->rsy[I],
           DZ = st->sz[I] - st->rsz[I];
    pbc(st, &DX, &DY, &DZ);
    if (DX * DX + DY * DY + DZ * DZ > h2) return 1;
  }
  return 0;
}

/* The list update of a step: every ICHNB-th step (reference), or when an
 * atom has moved half the skin (skin mode). */
static int list_due(ox_state *st, int MSTEP) {
  return st->p.rskin > 0. ? skin_moved(st) : MSTEP % st->p.ichnb == 0;
}

int ox_chcnb(ox_state *st, int32_t *mbsh, int32_t *mbln) {
  const int n = st->nstot;
  long capS = (long)st->caps * n, capL = (long)st->capl * n;
  long MBSH = 0, MBLN = 0;
  int iover = 0;
  int nth = st->nthreads;
  if (nth <= 1) {
    for (int I = 1; I <= n; ++I) {
      int imol = st->nnum[I];
      for (int J = I - 2; J >= 1; J -= 2) { /* even strip */
        int c = chcnb_pair(st, I, J, imol);
        if (c == 3) {
          if (MBSH < capS) { st->nbs1[MBSH + 1] = -I; st->nbs2[MBSH + 1] = J; }
          ++MBSH;
        } else if (c == 1) {
          if (MBSH < capS) { st->nbs1[MBSH + 1] = I; st->nbs2[MBSH + 1] = J; }
          ++MBSH;
        } else if (c == 2) {
          if (MBLN < capL) { st->nbl1[MBLN + 1] = I; st->nbl2[MBLN + 1] = J; }
          else iover = 1;
          ++MBLN;
        }
      }
      for (int J = I + 1; J <= n; J += 2) { /* odd strip */
        int c = chcnb_pair(st, I, J, imol);
        if (c == 3) {
          if (MBSH < capS) { st->nbs1[MBSH + 1] = -I; st->nbs2[MBSH + 1] = J; }
          ++MBSH;
        } else if (c == 1) {
          if (MBSH < capS) { st->nbs1[MBSH + 1] = J; st->nbs2[MBSH + 1] = I; }
          ++MBSH;
        } else if (c == 2) {
          if (MBLN < capL) { st->nbl1[MBLN + 1] = J; st->nbl2[MBLN + 1] = I; }
          else iover = 1;
          ++MBLN;
        }
      }
    }
  } else {
    /* Threads scan disjoint blocks of I into private buffers which are
     * concatenated in I order: the same lists as the serial scan. */
    int nblk = nth * 8;
    long *cs = (long *)xcalloc((size_t)nblk + 1, sizeof(long));
    long *cl = (long *)xcalloc((size_t)nblk + 1, sizeof(long));
    int **bs = (int **)xcalloc((size_t)nblk, sizeof(int *));
    int **bl = (int **)xcalloc((size_t)nblk, sizeof(int *));
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
    for (int b = 0; b < nblk; ++b) {
      int i0 = 1 + (int)((long)n * b / nblk), i1 = (int)((long)n * (b + 1) / nblk);
      long cap_s = 64, cap_l = 1024, ns = 0, nl = 0;
      int *ps = (int *)malloc(sizeof(int) * 2 * cap_s);
      int *pl = (int *)malloc(sizeof(int) * 2 * cap_l);
      for (int I = i0; I <= i1; ++I) {
        int imol = st->nnum[I];
        for (int pass = 0; pass < 2; ++pass) {
          int J = pass == 0 ? I - 2 : I + 1;
          int step = pass == 0 ? -2 : 2;
          for (; pass == 0 ? J >= 1 : J <= n; J += step) {
            int c = chcnb_pair(st, I, J, imol);
            if (c <= 0) continue;
            int a, bb;
            if (c == 3) { a = -I; bb = J; }
            else if (pass == 0) { a = I; bb = J; }
            else { a = J; bb = I; }
            if (c == 2) {
              if (nl == cap_l) { cap_l *= 2; pl = (int *)realloc(pl, sizeof(int) * 2 * cap_l); }
              pl[2 * nl] = a; pl[2 * nl + 1] = bb; ++nl;
            } else {
              if (ns == cap_s) { cap_s *= 2; ps = (int *)realloc(ps, sizeof(int) * 2 * cap_s); }
              ps[2 * ns] = a; ps[2 * ns + 1] = bb; ++ns;
            }
          }
        }
      }
      bs[b] = ps; bl[b] = pl; cs[b + 1] = ns; cl[b + 1] = nl;
    }
    for (int b = 0; b < nblk; ++b) {
      for (long k = 0; k < cs[b + 1]; ++k) {
        if (MBSH < capS) { st->nbs1[MBSH + 1] = bs[b][2 * k]; st->nbs2[MBSH + 1] = bs[b][2 * k + 1]; }
        ++MBSH;
      }
      for (long k = 0; k < cl[b + 1]; ++k) {
        if (MBLN < capL) { st->nbl1[MBLN + 1] = bl[b][2 * k]; st->nbl2[MBLN + 1] = bl[b][2 * k + 1]; }
        else iover = 1;
        ++MBLN;
      }
      free(bs[b]); free(bl[b]);
    }
    free(bs); free(bl); free(cs); free(cl);
  }
  st->mbsh = (int)(MBSH < capS ? MBSH : capS);
  st->mbln = (int)(MBLN < capL ? MBLN : capL);
  for (int I = 1; I <= n; ++I) {
    st->rsx[I] = st->sx[I];
    st->rsy[I] = st->sy[I];
    st->rsz[I] = st->sz[I];
  }
  st->nbuild++;
  if (mbsh) *mbsh = (int32_t)MBSH;
  if (mbln) *mbln = (int32_t)MBLN;
  if (MBSH > capS) {
    snprintf(st->msg, sizeof st->msg,
             "list of closest neighbours overfilled: %ld > %ld", MBSH, capS);
    return MDX_ERR_LIST_OVERFLOW;
  }
  if (iover || MBLN > capL) {
    snprintf(st->msg, sizeof st->msg,
             "list of far neighbours overfilled: need %ld > %ld", MBLN, capL);
    return MDX_ERR_LIST_OVERFLOW;
  }
  return MDX_OK;
}

int ox_get_lists(ox_state *st, int32_t *nbs1, int32_t *nbs2, int32_t cap_s,
                 int32_t *nbl1, int32_t *nbl2, int32_t cap_l) {
  if (st->mbsh > cap_s || st->mbln > cap_l) return MDX_ERR_ARG;
  for (int k = 0; k < st->mbsh; ++k) {
    nbs1[k] = st->nbs1[k + 1];
    nbs2[k] = st->nbs2[k + 1];
  }
  for (int k = 0; k < st->mbln; ++k) {
    nbl1[k] = st->nbl1[k + 1];
    nbl2[k] = st->nbl2[k + 1];
  }
  return MDX_OK;
}

/* --------------------------------------------------------------- ZEROFS */
static void zerofs(ox_state *st, int nnn) {
  mdx_scalars *s = &st->s;
  int molint = st->p.molint;
  if (nnn == 1) {
    s->pels2 = 0.; s->pint = 0.; s->pe2 = 0.; s->virb = 0.; s->vir2 = 0.;
    s->wirss = 0.; s->virfx = 0.; s->virfy = 0.; s->virfz = 0.;
    for (int i = 0; i < molint; ++i) { s->pote1[i] = 0.; s->potl1[i] = 0.; }
    for (int i = 0; i < st->ntypes; ++i) { s->pes141[i] = 0.; s->psr141[i] = 0.; }
    for (int i = 1; i <= st->nstot; ++i) { st->hx[i] = 0.; st->hy[i] = 0.; st->hz[i] = 0.; }
  } else {
    for (int i = 0; i < molint; ++i) { s->pote1[i] = 0.; s->potl1[i] = 0.; }
    for (int i = 0; i < st->ntypes; ++i) { s->pes141[i] = 0.; s->psr141[i] = 0.; }
    s->wirs = 0.; s->vir1 = 0.; s->pe1 = 0.; s->pels1 = 0.;
    s->virx = 0.; s->viry = 0.; s->virz = 0.;
    for (int i = 1; i <= st->nstot; ++i) { st->gx[i] = 0.; st->gy[i] = 0.; st->gz[i] = 0.; }
  }
}

/* Pair parameters common to LOCALF and FORCES (forces.f:838-862). */
static inline void pair_params(const ox_state *st, int ISP0, int ISP, int JSP,
                               double *QIJ, double *A6, double *B12,
                               double *RAE) {
  int ITYP = st->itype[ISP], JTYP = st->itype[JSP];
  int ISB = st->nsite[ISP], JSB = st->nsite[JSP];
  int IMOL = st->nnum[ISP], JMOL = st->nnum[JSP];
  int ISN = st->inbt[ISB], JSN = st->inbt[JSB];
  int nb = st->nnbt;
  if (IMOL == JMOL) {
    if (ISP0 < 0) {
      *QIJ = st->charge[ISB] * st->charge[JSB] * st->p.coulf * st->c14el[ITYP];
      *A6 = st->a6_14[IDX2(ISN, JSN, nb)] * st->c14lj[ITYP];
      *B12 = st->b12_14[IDX2(ISN, JSN, nb)] * st->c14lj[ITYP];
    } else {
      *QIJ = st->charge[ISB] * st->charge[JSB] * st->p.coulf;
      *A6 = st->a6lj0[IDX2(ISN, JSN, nb)];
      *B12 = st->b12lj0[IDX2(ISN, JSN, nb)];
    }
    *RAE = 0.;
  } else {
    *QIJ = st->q[ISP] * st->q[JSP] * st->p.coulf;
    *A6 = st->a6lj[IDX2(ISN, JSN, nb)];
    *B12 = st->b12lj[IDX2(ISN, JSN, nb)];
    *RAE = 0.;
    if (st->p.lmdee) {
      if (st->iee[ITYP] * st->iee[JTYP] == 0)
        *RAE = st->p.raex;
      else
        *RAE = 0.;
    }
  }
}

/* --------------------------------------------------------------- LOCALF */
static void localf_range(ox_state *st, mdx_scalars *s, double *hx, double *hy,
                         double *hz, int i0, int i1) {
  const double ALPHAD = st->p.alphad;
  for (int INP = i0; INP <= i1; ++INP) {
    int ISP0 = st->nbs1[INP];
    int ISP = abs(ISP0);
    int JSP = st->nbs2[INP];
    int ITYP = st->itype[ISP], JTYP = st->itype[JSP];
    int IMOL = st->nnum[ISP], JMOL = st->nnum[JSP];
    int MTR = st->mdxt[ITYP][JTYP];
    double QIJ, A6, B12, RAE;
    (void)JTYP;
    pair_params(st, ISP0, ISP, JSP, &QIJ, &A6, &B12, &RAE);
    double DX = st->sx[ISP] - st->sx[JSP];
    double DY = st->sy[ISP] - st->sy[JSP];
    double DZ = st->sz[ISP] - st->sz[JSP];
    pbc_h(st, &DX, &DY, &DZ, st->hboxl); /* forces.f:871 tests DZ vs HBOXL */
    double RR = DX * DX + DY * DY + DZ * DZ;
    double R1 = sqrt(RR);
    double R1I = 1. / R1;
    double R1E = R1 + RAE;
    double R1EI = 1. / R1E;
    double EE1, EES, FORCE;
    if (ISP0 <= 0 || (IMOL == JMOL && st->iee[ITYP] == 0)) {
      EE1 = QIJ * R1I;
      if (st->lmove[ITYP])
        FORCE = EE1 * (R1I * R1I);
      else
        FORCE = 0.;
      EES = EE1;
    } else if (st->p.lmnbl) {
      EE1 = QIJ * (1 / R1E - 0.5 * st->p.rff2 * (R1E * R1E) + st->p.rff);
      EES = EE1;
      FORCE = QIJ * (1. / (R1E * R1E * R1E) + st->p.rff2);
      s->vir2 = s->vir2 + QIJ * (1.5 * st->p.rff2 / (R1E * R1E) - st->p.rff);
    } else {
      double ALPHAR = ALPHAD * R1;
      double TTT = 1.0 / (1.0 + B1 * ALPHAR);
      double EXP2A = exp(-(ALPHAR * ALPHAR));
      double ERFCT = ((((A5 * TTT + A4) * TTT + A3) * TTT + A2) * TTT + A1) * TTT * EXP2A;
      EE1 = QIJ * R1EI;
      EES = EE1 * ERFCT;
      FORCE = EE1 * (TOTPI * ALPHAD * EXP2A + ERFCT * R1EI) * R1I;
    }
    if (IMOL == JMOL)
      s->pes141[ITYP - 1] = s->pes141[ITYP - 1] + EE1;
    else
      s->pote1[MTR - 1] = s->pote1[MTR - 1] + EE1;
    s->pels2 = s->pels2 + EES;
    if (B12 != 0.0) {
      double R2I = R1EI * R1EI;
      double R6I = R2I * R2I * R2I;
      double ESR = (A6 + B12 * R6I) * R6I;
      double FSR = (6.0 * A6 + 12.0 * B12 * R6I) * R6I * R1EI;
      FORCE = FORCE + FSR * R1I;
      if (IMOL == JMOL) {
        if (st->lmove[ITYP]) {
          s->psr141[ITYP - 1] = s->psr141[ITYP - 1] + ESR;
          s->vir2 = s->vir2 + FSR * R1;
        } else {
          ESR = 0.;
          FORCE = 0.;
        }
      } else {
        s->potl1[MTR - 1] = s->potl1[MTR - 1] + ESR;
        s->vir2 = s->vir2 + FSR * R1;
      }
      s->pe2 = s->pe2 + ESR;
    }
    hx[ISP] = hx[ISP] + FORCE * DX;
    hy[ISP] = hy[ISP] + FORCE * DY;
    hz[ISP] = hz[ISP] + FORCE * DZ;
    hx[JSP] = hx[JSP] - FORCE * DX;
    hy[JSP] = hy[JSP] - FORCE * DY;
    hz[JSP] = hz[JSP] - FORCE * DZ;
    s->virfx = s->virfx + FORCE * (DX * DX);
    s->virfy = s->virfy + FORCE * (DY * DY);
    s->virfz = s->virfz + FORCE * (DZ * DZ);
  }
}

/* Sum of thread-private accumulators of a parallel pair sweep (CPU baseline
 * runs only; the checker runs single-threaded in the reference's order). */
static void add_scalars(mdx_scalars *d, const mdx_scalars *a) {
  d->pe1 += a->pe1; d->pels1 += a->pels1; d->pe2 += a->pe2; d->pels2 += a->pels2;
  d->vir1 += a->vir1; d->vir2 += a->vir2;
  d->virx += a->virx; d->viry += a->viry; d->virz += a->virz;
  d->virfx += a->virfx; d->virfy += a->virfy; d->virfz += a->virfz;
  for (int k = 0; k < MDX_NTPP; ++k) { d->pote1[k] += a->pote1[k]; d->potl1[k] += a->potl1[k]; }
  for (int k = 0; k < MDX_NTPS; ++k) { d->pes141[k] += a->pes141[k]; d->psr141[k] += a->psr141[k]; }
}

typedef void (*pair_range_fn)(ox_state *, mdx_scalars *, double *, double *,
                              double *, int, int);

static void pair_sweep(ox_state *st, pair_range_fn fn, int npairs, double *fx,
                       double *fy, double *fz) {
  const int nth = st->nthreads;
  if (nth <= 1 || npairs < 10000) {
    fn(st, &st->s, fx, fy, fz, 1, npairs);
    return;
  }
  const int n = st->nstot;
  double *buf = (double *)xcalloc((size_t)nth * 3 * (n + 1), sizeof(double));
  mdx_scalars *ss = (mdx_scalars *)xcalloc((size_t)nth, sizeof(mdx_scalars));
#pragma omp parallel num_threads(nth)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    int i0 = 1 + (int)((long)npairs * t / nth), i1 = (int)((long)npairs * (t + 1) / nth);
    double *bx = buf + (size_t)t * 3 * (n + 1);
    fn(st, &ss[t], bx, bx + (n + 1), bx + 2 * (n + 1), i0, i1);
  }
  for (int t = 0; t < nth; ++t) {
    double *bx = buf + (size_t)t * 3 * (n + 1), *by = bx + (n + 1), *bz = by + (n + 1);
    for (int i = 1; i <= n; ++i) { fx[i] += bx[i]; fy[i] += by[i]; fz[i] += bz[i]; }
    add_scalars(&st->s, &ss[t]);
  }
  free(buf);
  free(ss);
}

static void localf(ox_state *st) {
  mdx_scalars *s = &st->s;
  pair_sweep(st, localf_range, st->mbsh, st->hx, st->hy, st->hz);
  for (int N = 1; N <= st->nstot; ++N) {
    int M = st->nnum[N];
    s->wirss = s->wirss - st->hx[N] * (st->sx[N] - st->X[M]) -
               st->hy[N] * (st->sy[N] - st->Y[M]) -
               st->hz[N] * (st->sz[N] - st->Z[M]);
  }
}

/* --------------------------------------------------------------- FORCES */
static void forces_range(ox_state *st, mdx_scalars *s, double *gx, double *gy,
                         double *gz, int i0, int i1) {
  const double ALPHAD = st->p.alphad;
  for (int INP = i0; INP <= i1; ++INP) {
    int ISP0 = st->nbl1[INP];
    int JSP = st->nbl2[INP];
    int ISP = abs(ISP0);
    int ITYP = st->itype[ISP], JTYP = st->itype[JSP];
    int IMOL = st->nnum[ISP], JMOL = st->nnum[JSP];
    int MTR = st->mdxt[ITYP][JTYP];
    double QIJ, A6, B12, RAE;
    pair_params(st, ISP0, ISP, JSP, &QIJ, &A6, &B12, &RAE);
    double DX = st->sx[ISP] - st->sx[JSP];
    double DY = st->sy[ISP] - st->sy[JSP];
    double DZ = st->sz[ISP] - st->sz[JSP];
    pbc(st, &DX, &DY, &DZ);
    double RR = DX * DX + DY * DY + DZ * DZ;
    /* skin mode: the list reaches RCUT + skin, pairs beyond RCUT are skipped */
    if (st->p.rskin > 0. && RR > st->rssq) continue;
    double R1 = sqrt(RR);
    double R1I = 1. / R1;
    double R1E = R1 + RAE;
    double R1EI = 1. / R1E;
    double EE1, EES, FORCE;
    (void)R1I;
    if (ISP0 <= 0 || (IMOL == JMOL && st->iee[ITYP] == 0)) {
      EE1 = QIJ / R1;
      if (st->lmove[ITYP])
        FORCE = EE1 / (R1 * R1);
      else
        FORCE = 0.;
      EES = EE1;
    } else if (st->p.lmnbl) {
      EE1 = QIJ * (1 / R1E - 0.5 * st->p.rff2 * (R1E * R1E) + st->p.rff);
      EES = EE1;
      FORCE = QIJ * (1 / ((R1E * R1E) * R1) + st->p.rff2);
      s->vir1 = s->vir1 + QIJ * (1.5 * st->p.rff2 * RR - st->p.rff);
    } else {
      double ALPHAR = ALPHAD * R1;
      double TTT = 1.0 / (1.0 + B1 * ALPHAR);
      double EXP2A = exp(-(ALPHAR * ALPHAR));
      double ERFCT = ((((A5 * TTT + A4) * TTT + A3) * TTT + A2) * TTT + A1) * TTT * EXP2A;
      EE1 = QIJ * R1EI;
      EES = EE1 * ERFCT;
      FORCE = EE1 * (TOTPI * ALPHAD * EXP2A + ERFCT * R1EI) * R1I;
    }
    if (IMOL == JMOL)
      s->pes141[ITYP - 1] = s->pes141[ITYP - 1] + EE1;
    else
      s->pote1[MTR - 1] = s->pote1[MTR - 1] + EE1;
    s->pels1 = s->pels1 + EES;
    if (B12 != 0.0) {
      double R2I = R1EI * R1EI;
      double R6I = R2I * R2I * R2I;
      double ESR = (A6 + B12 * R6I) * R6I;
      double FSR = (6.0 * A6 + 12.0 * B12 * R6I) * R6I * R1EI;
      FORCE = FORCE + FSR * R1I;
      if (IMOL == JMOL) {
        if (st->lmove[ITYP]) s->vir1 = s->vir1 + FSR * R1;
        s->psr141[ITYP - 1] = s->psr141[ITYP - 1] + ESR;
      } else {
        s->potl1[MTR - 1] = s->potl1[MTR - 1] + ESR;
        s->vir1 = s->vir1 + FSR * R1;
      }
      s->pe1 = s->pe1 + ESR;
    }
    if (IMOL != JMOL || st->lmove[ITYP]) {
      s->virx = s->virx + FORCE * (DX * DX);
      s->viry = s->viry + FORCE * (DY * DY);
      s->virz = s->virz + FORCE * (DZ * DZ);
    }
    gx[ISP] = gx[ISP] + FORCE * DX;
    gy[ISP] = gy[ISP] + FORCE * DY;
    gz[ISP] = gz[ISP] + FORCE * DZ;
    gx[JSP] = gx[JSP] - FORCE * DX;
    gy[JSP] = gy[JSP] - FORCE * DY;
    gz[JSP] = gz[JSP] - FORCE * DZ;
  }
}

static void forces_long(ox_state *st) {
  pair_sweep(st, forces_range, st->mbln, st->gx, st->gy, st->gz);
}

/* ---------------------------------------------------------------- INIFUR */
int ox_inifur(ox_state *st, int32_t *nkv) {
  double ALP2 = st->p.alphad * st->p.alphad;
  double CUTK2 = 4.0 * ALP2 * st->p.fexp;
  double CUTK = sqrt(CUTK2);
  double TWOPI = 2.0 * PI;
  int IKV = 0;
  int KMAX = (int)(CUTK * st->boxl / TWOPI + 1);
  int KMAY = (int)(CUTK * st->boyl / TWOPI + 1);
  int KMAZ = (int)(CUTK * st->bozl / TWOPI + 1);
  for (int IKZ = -KMAZ; IKZ <= KMAZ; ++IKZ)
    for (int IKX = 0; IKX <= KMAX; ++IKX) {
      int KY1, KY2;
      if (IKX == 0) {
        KY1 = IKZ > 0 ? 0 : 1;
        KY2 = KMAY;
      } else {
        KY1 = -KMAY;
        KY2 = KMAY;
      }
      for (int IKY = KY1; IKY <= KY2; ++IKY) {
        double RXV, RYV, RZV;
        if (st->p.icell == 1) {
          RXV = TWOPI * IKX; RYV = TWOPI * IKY; RZV = TWOPI * (-IKX + IKY + 2 * IKZ);
        } else if (st->p.icell == 2) {
          RXV = TWOPI * IKX; RYV = TWOPI * IKY + PI * IKX; RZV = TWOPI * IKZ;
        } else {
          RXV = TWOPI * IKX; RYV = TWOPI * IKY; RZV = TWOPI * IKZ;
        }
        double rx = RXV / st->boxl, ry = RYV / st->boyl, rz = RZV / st->bozl;
        double RK2 = rx * rx + ry * ry + rz * rz;
        if (RK2 <= CUTK2) {
          IKV = IKV + 1;
          if (IKV > st->nkvm) {
            snprintf(st->msg, sizeof st->msg, "max number of reciprocal vectors exceeded");
            return MDX_ERR_KVEC;
          }
          st->rkx[IKV] = RXV;
          st->rky[IKV] = RYV;
          st->rkz[IKV] = RZV;
        }
      }
    }
  st->nkv = IKV;
  double ABC = st->p.alphad / sqrt(PI);
  st->spei = 0.;
  for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP) {
    double SPET = 0.;
    double ESCI = st->iee[ITYP] == 0 ? st->p.ec_me : 1.0;
    for (int I = 1; I <= st->nsits[ITYP]; ++I) {
      int IS = st->isadr[ITYP] + I;
      double eq = ESCI * st->charge[IS];
      double QII = st->p.coulf * (eq * eq);
      SPET = SPET - st->nspec[ITYP] * ABC * QII;
    }
    st->speei[ITYP] = SPET;
    st->spei = st->spei + SPET;
  }
  if (nkv) *nkv = IKV;
  return MDX_OK;
}

/* ----------------------------------------------------------------- FURIR */
static int furir(ox_state *st) {
  const double FKTX = 1.05, FKTS = 0.95;
  mdx_scalars *s = &st->s;
  int rc;
  if (!st->furir_init) {
    st->furir_init = 1;
    st->boxlo = st->boxl;
    st->boylo = st->boyl;
    st->bozlo = st->bozl;
    if (st->p.alphad > 0.0) {
      if ((rc = ox_inifur(st, NULL))) return rc;
    } else {
      st->nkv = 0;
    }
  }
  double DBX = st->boxl / st->boxlo, DBY = st->boyl / st->boylo, DBZ = st->bozl / st->bozlo;
  if (DBX > FKTX || DBX < FKTS || DBY > FKTX || DBY < FKTS || DBZ > FKTX || DBZ < FKTS) {
    st->boxlo = st->boxl;
    st->boylo = st->boyl;
    st->bozlo = st->bozl;
    if ((rc = ox_inifur(st, NULL))) return rc;
  }
  s->nkv = st->nkv;
  if (st->nkv == 0 || (st->ntypes == 1 && st->nspec[1] == 1)) return MDX_OK;
  const double ALP2 = st->p.alphad * st->p.alphad;
  const double CFUR = 4.0 * PI * st->p.coulf / st->vol;
  const int n = st->nstot;
  double QPE = 0.0, vx_ = 0., vy_ = 0., vz_ = 0.;
  int nth = st->nthreads;
  if (nth <= 1) {
    double *TSIN = (double *)xcalloc((size_t)n + 1, sizeof(double));
    double *TCOS = (double *)xcalloc((size_t)n + 1, sizeof(double));
    for (int IKV = 1; IKV <= st->nkv; ++IKV) {
      double RXV = st->rkx[IKV] / st->boxl;
      double RYV = st->rky[IKV] / st->boyl;
      double RZV = st->rkz[IKV] / st->bozl;
      double RK2 = RXV * RXV + RYV * RYV + RZV * RZV;
      double SCS = 0., SSN = 0.;
      for (int I = 1; I <= n; ++I) {
        double SCP = RXV * st->sx[I] + RYV * st->sy[I] + RZV * st->sz[I];
        double QQ = st->q[I];
        double SINSC = QQ * sin(SCP);
        double COSSC = QQ * cos(SCP);
        TSIN[I] = SINSC;
        TCOS[I] = COSSC;
        SSN = SSN + SINSC;
        SCS = SCS + COSSC;
      }
      double AKC = CFUR * exp(-0.25 * RK2 / ALP2) / RK2;
      QPE = QPE + AKC * (SSN * SSN + SCS * SCS);
      double AK2 = 2.0 * AKC;
      for (int I = 1; I <= n; ++I) {
        double QFOR = AK2 * (SCS * TSIN[I] - SSN * TCOS[I]);
        st->gx[I] = st->gx[I] + RXV * QFOR;
        st->gy[I] = st->gy[I] + RYV * QFOR;
        st->gz[I] = st->gz[I] + RZV * QFOR;
      }
      double AKV = 0.5 * AKC * (4. * ALP2 + RK2) / (ALP2 * RK2);
      double S2 = SSN * SSN + SCS * SCS;
      s->virx = s->virx - (RXV * RXV) * AKV * S2;
      s->viry = s->viry - (RYV * RYV) * AKV * S2;
      s->virz = s->virz - (RZV * RZV) * AKV * S2;
    }
    free(TSIN);
    free(TCOS);
  } else {
    /* threads take disjoint k ranges with private force buffers */
    double *gacc = (double *)xcalloc((size_t)nth * 3 * (n + 1), sizeof(double));
    double *eacc = (double *)xcalloc((size_t)nth * 4, sizeof(double));
#pragma omp parallel num_threads(nth)
    {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      double *gx = gacc + (size_t)tid * 3 * (n + 1), *gy = gx + (n + 1), *gz = gy + (n + 1);
      double *TSIN = (double *)malloc(sizeof(double) * (n + 1));
      double *TCOS = (double *)malloc(sizeof(double) * (n + 1));
      double qpe = 0., v1 = 0., v2 = 0., v3 = 0.;
#pragma omp for schedule(static)
      for (int IKV = 1; IKV <= st->nkv; ++IKV) {
        double RXV = st->rkx[IKV] / st->boxl, RYV = st->rky[IKV] / st->boyl, RZV = st->rkz[IKV] / st->bozl;
        double RK2 = RXV * RXV + RYV * RYV + RZV * RZV;
        double SCS = 0., SSN = 0.;
        for (int I = 1; I <= n; ++I) {
          double SCP = RXV * st->sx[I] + RYV * st->sy[I] + RZV * st->sz[I];
          double QQ = st->q[I];
          TSIN[I] = QQ * sin(SCP);
          TCOS[I] = QQ * cos(SCP);
          SSN += TSIN[I];
          SCS += TCOS[I];
        }
        double AKC = CFUR * exp(-0.25 * RK2 / ALP2) / RK2;
        qpe += AKC * (SSN * SSN + SCS * SCS);
        double AK2 = 2.0 * AKC;
        for (int I = 1; I <= n; ++I) {
          double QFOR = AK2 * (SCS * TSIN[I] - SSN * TCOS[I]);
          gx[I] += RXV * QFOR; gy[I] += RYV * QFOR; gz[I] += RZV * QFOR;
        }
        double AKV = 0.5 * AKC * (4. * ALP2 + RK2) / (ALP2 * RK2);
        double S2 = SSN * SSN + SCS * SCS;
        v1 -= RXV * RXV * AKV * S2; v2 -= RYV * RYV * AKV * S2; v3 -= RZV * RZV * AKV * S2;
      }
      eacc[4 * tid] = qpe; eacc[4 * tid + 1] = v1; eacc[4 * tid + 2] = v2; eacc[4 * tid + 3] = v3;
      free(TSIN); free(TCOS);
    }
    for (int t = 0; t < nth; ++t) {
      double *gx = gacc + (size_t)t * 3 * (n + 1), *gy = gx + (n + 1), *gz = gy + (n + 1);
      for (int I = 1; I <= n; ++I) { st->gx[I] += gx[I]; st->gy[I] += gy[I]; st->gz[I] += gz[I]; }
      QPE += eacc[4 * t]; vx_ += eacc[4 * t + 1]; vy_ += eacc[4 * t + 2]; vz_ += eacc[4 * t + 3];
    }
    s->virx += vx_; s->viry += vy_; s->virz += vz_;
    free(gacc); free(eacc);
  }
  s->virx = s->virx + QPE;
  s->viry = s->viry + QPE;
  s->virz = s->virz + QPE;
  s->pels1 = s->pels1 + QPE;
  s->qpe = QPE;
  return MDX_OK;
}

/* ---------------------------------------------------------------- ETERMS */
static void eterms_pair(ox_state *st, int ISP, int JSP, int ITYP) {
  mdx_scalars *s = &st->s;
  const double ALPHAD = st->p.alphad;
  double QIJ = st->p.coulf * st->q[ISP] * st->q[JSP];
  double DX = st->sx[ISP] - st->sx[JSP];
  double DY = st->sy[ISP] - st->sy[JSP];
  double DZ = st->sz[ISP] - st->sz[JSP];
  pbc(st, &DX, &DY, &DZ);
  double R2 = DX * DX + DY * DY + DZ * DZ;
  double R2I = 1.0 / R2;
  double R1 = sqrt(R2);
  double R1I = R1 * R2I;
  double ALPHAR = ALPHAD * R1;
  double TTT = 1.0 / (1.0 + B1 * ALPHAR);
  double EXP2A = exp(-(ALPHAR * ALPHAR));
  double ERFC = ((((A5 * TTT + A4) * TTT + A3) * TTT + A2) * TTT + A1) * TTT * EXP2A;
  double EES = QIJ * (ERFC - 1.0) * R1I;
  s->spe = s->spe + EES;
  s->spee[ITYP - 1] = s->spee[ITYP - 1] + EES;
  if (st->lmove[ITYP]) {
    double FES = QIJ * ((TOTPI * ALPHAR * EXP2A + ERFC) - 1.0) * R1I * R2I;
    st->gx[ISP] = st->gx[ISP] + FES * DX;
    st->gy[ISP] = st->gy[ISP] + FES * DY;
    st->gz[ISP] = st->gz[ISP] + FES * DZ;
    st->gx[JSP] = st->gx[JSP] - FES * DX;
    st->gy[JSP] = st->gy[JSP] - FES * DY;
    st->gz[JSP] = st->gz[JSP] - FES * DZ;
    s->virx = s->virx + FES * (DX * DX);
    s->viry = s->viry + FES * (DY * DY);
    s->virz = s->virz + FES * (DZ * DZ);
  }
}

static void eterms(ox_state *st) {
  mdx_scalars *s = &st->s;
  if (st->p.lmnbl) return;
  for (int I = 1; I <= st->ntypes; ++I) s->spee[I - 1] = st->speei[I];
  s->spe = st->spei;
  for (int ISP = 1; ISP <= st->nstot; ++ISP) {
    int ITYP = st->itype[ISP];
    if (st->iee[ITYP] != 0) {
      int NSP = st->nnbb[ISP];
      for (int J = 1; J <= NSP; ++J) {
        int JSP = st->inbb[IDX2(ISP, J, st->nstot)];
        if (JSP <= 0) JSP = -JSP;
        if (ISP > JSP) eterms_pair(st, ISP, JSP, ITYP);
      }
    }
  }
  for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP) {
    if (st->iee[ITYP] == 0) {
      for (int IM = 0; IM <= st->nspec[ITYP] - 1; ++IM) {
        int NSP = st->nsits[ITYP];
        int ISPI = st->isaddr[ITYP] + NSP * IM;
        if (NSP > 1)
          for (int ISM = 2; ISM <= NSP; ++ISM)
            for (int JSM = 1; JSM <= ISM - 1; ++JSM)
              eterms_pair(st, ISPI + ISM, ISPI + JSM, ITYP);
      }
    }
  }
}

/* ---------------------------------------------------------------- GETBND */
static void strbnd(ox_state *st, int ITYP);

static void getbnd(ox_state *st) {
  mdx_scalars *s = &st->s;
  for (int M = 1; M <= st->nrbb; ++M) {
    st->br[M] = 0.;
    st->be[M] = 0.;
  }
  for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP)
    if (st->ipot[ITYP] == 1 || st->ipot[ITYP] == 2) strbnd(st, ITYP);
  if (st->nrbb <= 0) return;
  for (int N = 1; N <= st->nrbt; ++N) {
    int I = st->ibi[N];
    int ITYP = st->itype[I];
    int M = st->ibuk[N];
    int J = st->jbj[N];
    int NSP = st->nspec[ITYP];
    double FNSPI = 1.0 / (double)NSP;
    double REQ = st->rb[M];
    double BX = st->sx[J] - st->sx[I];
    double BY = st->sy[J] - st->sy[I];
    double BZ = st->sz[J] - st->sz[I];
    pbc(st, &BX, &BY, &BZ);
    double BSQ = BX * BX + BY * BY + BZ * BZ;
    double BD = sqrt(BSQ);
    double R1I = 1.0 / BD;
    double BBB = BD - REQ;
    double EBDD, FORB;
    if (st->id[M] != 1 || BBB > REQ) {
      double FCN = st->fb[M];
      double DBND = BBB * FCN;
      EBDD = DBND * BBB;
      FORB = -2.0 * DBND * R1I;
    } else {
      double DDIS = st->db[M];
      double ROH = st->ro[M];
      double EXM = exp(-ROH * BBB);
      double EXMP = 1 - EXM;
      EBDD = DDIS * (EXMP * EXMP);
      FORB = -2.0 * DDIS * ROH * EXM * EXMP * R1I;
    }
    st->br[M] = st->br[M] + BD * FNSPI;
    st->be[M] = st->be[M] + EBDD * FNSPI;
    s->pint = s->pint + EBDD;
    if (st->lmove[ITYP]) {
      st->hx[I] = st->hx[I] - BX * FORB;
      st->hy[I] = st->hy[I] - BY * FORB;
      st->hz[I] = st->hz[I] - BZ * FORB;
      st->hx[J] = st->hx[J] + BX * FORB;
      st->hy[J] = st->hy[J] + BY * FORB;
      st->hz[J] = st->hz[J] + BZ * FORB;
      s->virb = s->virb + FORB * BSQ;
      s->virfx = s->virfx + FORB * (BX * BX);
      s->virfy = s->virfy + FORB * (BY * BY);
      s->virfz = s->virfz + FORB * (BZ * BZ);
    }
  }
}

/* ---------------------------------------------------------------- GETANG */
static void getang(ox_state *st) {
  mdx_scalars *s = &st->s;
  if (st->nraa <= 0) return;
  for (int M = 1; M <= st->nraa; ++M) {
    st->ar[M] = 0.;
    st->ae[M] = 0.;
  }
  for (int N = 1; N <= st->nrat; ++N) {
    int I = st->iai[N];
    int ITYP = st->itype[I];
    int J = st->jaj[N];
    int K = st->kak[N];
    int M = st->iauk[N];
    double FCN = st->fa[M];
    double AEQ = st->ra[M];
    int NSP = st->nspec[ITYP];
    double FNSPI = 1.0 / (double)NSP;
    double AX = st->sx[I] - st->sx[J];
    double AY = st->sy[I] - st->sy[J];
    double AZ = st->sz[I] - st->sz[J];
    pbc(st, &AX, &AY, &AZ);
    double ASQ = AX * AX + AY * AY + AZ * AZ;
    double ASQI = 1.0 / ASQ;
    double BX = st->sx[K] - st->sx[J];
    double BY = st->sy[K] - st->sy[J];
    double BZ = st->sz[K] - st->sz[J];
    pbc(st, &BX, &BY, &BZ);
    double BSQ = BX * BX + BY * BY + BZ * BZ;
    double BSQI = 1.0 / BSQ;
    double AB = sqrt(ASQ * BSQ);
    double ABI = 1.0 / AB;
    double COSA = AX * BX + AY * BY + AZ * BZ;
    COSA = COSA * ABI;
    COSA = fmin(COSA, 1.0);
    COSA = fmax(COSA, -1.0);
    double ALF = acos(COSA);
    double SINA = sin(ALF);
    double SINAI = 1.0 / SINA;
    double DALF = ALF - AEQ;
    double ABC = DALF * FCN;
    double EANG = ABC * DALF;
    st->ar[M] = st->ar[M] + ALF * FNSPI;
    st->ae[M] = st->ae[M] + EANG * FNSPI;
    s->pint = s->pint + EANG;
    if (st->lmove[ITYP]) {
      double SAB = -2.0 * ABC * SINAI;
      double CAB = SAB * COSA;
      double FAB = SAB * ABI;
      double FAA = CAB * ASQI;
      double FBB = CAB * BSQI;
      double FAX = FAB * BX - FAA * AX;
      double FAY = FAB * BY - FAA * AY;
      double FAZ = FAB * BZ - FAA * AZ;
      double FBX = FAB * AX - FBB * BX;
      double FBY = FAB * AY - FBB * BY;
      double FBZ = FAB * AZ - FBB * BZ;
      st->hx[I] = st->hx[I] - FAX;
      st->hy[I] = st->hy[I] - FAY;
      st->hz[I] = st->hz[I] - FAZ;
      st->hx[J] = st->hx[J] + FAX + FBX;
      st->hy[J] = st->hy[J] + FAY + FBY;
      st->hz[J] = st->hz[J] + FAZ + FBZ;
      st->hx[K] = st->hx[K] - FBX;
      st->hy[K] = st->hy[K] - FBY;
      st->hz[K] = st->hz[K] - FBZ;
      s->virfx = s->virfx - AX * FAX - BX * FBX;
      s->virfy = s->virfy - AY * FAY - BY * FBY;
      s->virfz = s->virfz - AZ * FAZ - BZ * FBZ;
    }
  }
}

/* ---------------------------------------------------------------- GETTRS */
static void gettrs(ox_state *st) {
  mdx_scalars *s = &st->s;
  if (st->nrtt <= 0) return;
  for (int M = 1; M <= st->nrtt; ++M) {
    st->tr[M] = 0.;
    st->te[M] = 0.;
  }
  for (int N = 1; N <= st->nrrt; ++N) {
    int I = st->iti[N], ITYP = st->itype[I];
    int J = st->jtj[N], K = st->ktk[N], L = st->ltl[N], M = st->ituk[N];
    int NSP = st->nspec[ITYP];
    double FNSPI = 1.0 / (double)NSP;
    double ax = st->sx[J] - st->sx[I], ay = st->sy[J] - st->sy[I], az = st->sz[J] - st->sz[I];
    double bx = st->sx[K] - st->sx[J], by = st->sy[K] - st->sy[J], bz = st->sz[K] - st->sz[J];
    double cx = st->sx[L] - st->sx[K], cy = st->sy[L] - st->sy[K], cz = st->sz[L] - st->sz[K];
    pbc(st, &ax, &ay, &az);
    pbc(st, &bx, &by, &bz);
    pbc(st, &cx, &cy, &cz);
    double ab = ax * bx + ay * by + az * bz;
    double bc = bx * cx + by * cy + bz * cz;
    double ac = ax * cx + ay * cy + az * cz;
    double at = ax * ax + ay * ay + az * az;
    double bt = bx * bx + by * by + bz * bz;
    double ct = cx * cx + cy * cy + cz * cz;
    double axb = (at * bt) - (ab * ab);
    double bxc = (bt * ct) - (bc * bc);
    double fnum = (ab * bc) - (ac * bt);
    double den = axb * bxc;
    if (!(den > 1.0e-10)) continue;
    den = sqrt(den);
    double co = fnum / den;
    co = fmin(co, 1.0);
    co = fmax(co, -1.0);
    double signum = ax * (by * cz - cy * bz) + ay * (bz * cx - cz * bx) + az * (bx * cy - cx * by);
    double arg = sgn(acos(co), signum);
    double SIN1F = sin(arg);
    double si = SIN1F;
    if (fabs(si) < 1.0e-10) si = sgn(1.0e-10, si);
    double POTT, DERI;
    int it = st->itors[M];
    if (it == 0) {
      double FCN = st->ft[M], TEQ = st->rt[M];
      int MUL = st->nmul[M];
      double EARG = MUL * arg - TEQ;
      POTT = FCN * (1.0 + cos(EARG));
      DERI = -FCN * MUL * sin(EARG);
    } else if (it == 1) {
      double FN1 = st->ft1[M], FN2 = st->ft2[M], FN3 = st->ft3[M];
      double COS1F = cos(arg);
      double COS2F = 2.0 * (COS1F * COS1F) - 1.0;
      double COS3F = COS1F * (2.0 * COS2F - 1.0);
      double SIN2F = 2.0 * SIN1F * COS1F;
      double SIN3F = SIN1F * COS2F + SIN2F * COS1F;
      POTT = FN1 * (1.0 + COS1F) + FN2 * (1.0 - COS2F) + FN3 * (1.0 + COS3F);
      DERI = -FN1 * SIN1F + 2.0 * FN2 * SIN2F - 3.0 * FN3 * SIN3F;
    } else if (it == 5) {
      double FN0 = st->ft[M], FN1 = st->ft1[M], FN2 = st->ft2[M], FN3 = st->ft3[M],
             FN4 = st->ft4[M], FN5 = st->ft5[M], TEQ = st->rt[M];
      double EARG = arg - TEQ;
      double COSI = cos(EARG);
      double COSI2 = COSI * COSI, COSI3 = COSI * COSI2, COSI4 = COSI * COSI3, COSI5 = COSI * COSI4;
      double SINI = sin(EARG);
      POTT = FN0 + FN1 * COSI + FN2 * COSI2 + FN3 * COSI3 + FN4 * COSI4 + FN5 * COSI5;
      DERI = -SINI * (FN1 + 2.0 * FN2 * COSI + 3.0 * FN3 * COSI2 + 4.0 * FN4 * COSI3 +
                      5.0 * FN5 * COSI4);
    } else if (it == -1) {
      double FCN = st->ft[M], TEQ = st->rt[M];
      double EARG = arg - TEQ;
      POTT = FCN * (EARG * EARG);
      DERI = 2.0 * FCN * EARG;
    } else {
      continue;
    }
    st->tr[M] = st->tr[M] + fabs(arg * FNSPI);
    st->te[M] = st->te[M] + POTT * FNSPI;
    s->pint = s->pint + POTT;
    if (st->lmove[ITYP]) {
      double de1 = DERI / den / si;
      axb = axb / den * co;
      bxc = bxc / den * co;
      double dnum, dden;
      dnum = cx * bt - bx * bc;
      dden = (ab * bx - ax * bt) * bxc;
      double FFI1 = (dnum - dden) * de1;
      dnum = ((bx - ax) * bc - ab * cx) + (2.0 * ac * bx - cx * bt);
      dden = axb * (bc * cx - bx * ct) + (ax * bt - at * bx - ab * (bx - ax)) * bxc;
      double FFJ1 = (dnum - dden) * de1;
      dnum = ab * bx - ax * bt;
      dden = axb * (bt * cx - bc * bx);
      double FFL1 = (dnum - dden) * de1;
      double FFK1 = -(FFI1 + FFJ1 + FFL1);
      st->hx[I] += FFI1; st->hx[J] += FFJ1; st->hx[K] += FFK1; st->hx[L] += FFL1;
      dnum = cy * bt - by * bc;
      dden = (ab * by - ay * bt) * bxc;
      double FFI2 = (dnum - dden) * de1;
      dnum = ((by - ay) * bc - ab * cy) + (2.0 * ac * by - cy * bt);
      dden = axb * (bc * cy - by * ct) + (ay * bt - at * by - ab * (by - ay)) * bxc;
      double FFJ2 = (dnum - dden) * de1;
      dnum = ab * by - ay * bt;
      dden = axb * (bt * cy - bc * by);
      double FFL2 = (dnum - dden) * de1;
      double FFK2 = -(FFI2 + FFJ2 + FFL2);
      st->hy[I] += FFI2; st->hy[J] += FFJ2; st->hy[K] += FFK2; st->hy[L] += FFL2;
      dnum = cz * bt - bz * bc;
      dden = (ab * bz - az * bt) * bxc;
      double FFI3 = (dnum - dden) * de1;
      dnum = ((bz - az) * bc - ab * cz) + (2.0 * ac * bz - cz * bt);
      dden = axb * (bc * cz - bz * ct) + (az * bt - at * bz - ab * (bz - az)) * bxc;
      double FFJ3 = (dnum - dden) * de1;
      dnum = ab * bz - az * bt;
      dden = axb * (bt * cz - bc * bz);
      double FFL3 = (dnum - dden) * de1;
      double FFK3 = -(FFI3 + FFJ3 + FFL3);
      st->hz[I] += FFI3; st->hz[J] += FFJ3; st->hz[K] += FFK3; st->hz[L] += FFL3;
      s->virfx = s->virfx - (ax + bx) * FFI1 - bx * FFJ1 + cx * FFL1;
      s->virfy = s->virfy - (ay + by) * FFI2 - by * FFJ2 + cy * FFL2;
      s->virfz = s->virfz - (az + bz) * FFI3 - bz * FFJ3 + cz * FFL3;
    }
  }
}

/* ---------------------------------------------------------------- STRBND */
static void strbnd(ox_state *st, int ITYP) {
  mdx_scalars *s = &st->s;
  const double EEP = -884.63, GGP = 467.31;
  const double BBMA = (double)1.3f, BBSA = (double)1.4f;
  int I1 = st->iadb[ITYP], I2 = I1 + 1, I3 = I2 + 1;
  int NSP = st->nspec[ITYP], NSS = st->nsits[ITYP];
  double FNSPI = 1.0 / (double)NSP;
  double ROH1 = st->rb[I1], ROH2 = st->rb[I2], RH1H2 = st->rb[I3];
  const double FACTOR = st->p.efact; /* 1.D3/AVSNO/UNITE, forces.f:593 */
  int IPT = st->ipot[ITYP];
  double AAA, BBB;
  if (IPT == 2) {
    AAA = st->db[I1];
    BBB = st->db[I2];
  } else {
    AAA = st->fb[I1];
    BBB = st->fb[I2];
  }
  double CCC = st->fb[I3];
  double EEE = EEP * FACTOR;
  double FFF = EEP * FACTOR;
  double GGG = GGP * FACTOR;
  double BBM = BBMA, BBS = BBSA;
  double AADD = AAA * st->ro[I1];
  double BBDD = BBB * st->ro[I2];
  int ISHF = st->isaddr[ITYP];
  int IBB = ISHF + 1, JBB = ISHF + 2, KBB = ISHF + 3;
  for (int N = 1; N <= NSP; ++N) {
    int I = (N - 1) * NSS + IBB, J = (N - 1) * NSS + JBB, K = (N - 1) * NSS + KBB;
    double AX = st->sx[J] - st->sx[I], AY = st->sy[J] - st->sy[I], AZ = st->sz[J] - st->sz[I];
    double BX = st->sx[K] - st->sx[I], BY = st->sy[K] - st->sy[I], BZ = st->sz[K] - st->sz[I];
    double CX = st->sx[K] - st->sx[J], CY = st->sy[K] - st->sy[J], CZ = st->sz[K] - st->sz[J];
    if (IPT == 2) {
      pbc(st, &AX, &AY, &AZ);
      pbc(st, &BX, &BY, &BZ);
      pbc(st, &CX, &CY, &CZ);
    }
    double RRA = AX * AX + AY * AY + AZ * AZ;
    double RRB = BX * BX + BY * BY + BZ * BZ;
    double RRC = CX * CX + CY * CY + CZ * CZ;
    double ASS = sqrt(RRA), BSS = sqrt(RRB), CSS = sqrt(RRC);
    double SA = ASS - ROH1, SB = BSS - ROH2, SH = CSS - RH1H2;
    double WB1, WB2, WB3, FB3A, FB3B, FB3C;
    if (IPT == 2) {
      double EXPA = exp(-st->ro[I1] * SA);
      double EXPAM = 1.0 - EXPA;
      double EXPB = exp(-st->ro[I2] * SB);
      double EXPBM = 1.0 - EXPB;
      WB1 = AAA * (EXPAM * EXPAM) + EEE * SA * SH;
      WB2 = BBB * (EXPBM * EXPBM) + FFF * SB * SH;
      WB3 = CCC * SH * SH + GGG * SA * SB;
    } else {
      WB1 = AAA * SA * SA + EEE * SA * SH;
      WB2 = BBB * SB * SB + FFF * SB * SH;
      WB3 = CCC * SH * SH + GGG * SA * SB;
    }
    st->br[I1] += ASS * FNSPI;
    st->br[I2] += BSS * FNSPI;
    st->br[I3] += CSS * FNSPI;
    st->be[I1] += WB1 * FNSPI;
    st->be[I2] += WB2 * FNSPI;
    st->be[I3] += WB3 * FNSPI;
    s->pint = s->pint + WB1 + WB2 + WB3;
    if (!st->lmove[ITYP]) continue;
    if (IPT == 2) {
      double EXPA = exp(-st->ro[I1] * SA), EXPAM = 1.0 - EXPA;
      double EXPB = exp(-st->ro[I2] * SB), EXPBM = 1.0 - EXPB;
      if (ASS > BBM)
        FB3A = -2. * SA * AADD * st->ro[I1];
      else
        FB3A = -2. * AADD * EXPA * EXPAM;
      FB3A = FB3A - EEE * SH - GGG * SB;
      if (BSS > BBM)
        FB3B = -2. * SB * BBDD * st->ro[I1];
      else
        FB3B = -2. * BBDD * EXPB * EXPBM;
      FB3B = FB3B - FFF * SH - GGG * SA;
      FB3C = -2.0 * CCC * SH - EEE * SA - FFF * SB;
    } else {
      FB3A = -2.0 * AAA * SA - EEE * SH - GGG * SB;
      FB3B = -2.0 * BBB * SB - FFF * SH - GGG * SA;
      FB3C = -2.0 * CCC * SH - EEE * SA - FFF * SB;
    }
    (void)BBS;
    FB3A = FB3A / ASS;
    FB3B = FB3B / BSS;
    FB3C = FB3C / CSS;
    double AXX = FB3A * AX, AYY = FB3A * AY, AZZ = FB3A * AZ;
    double BXX = FB3B * BX, BYY = FB3B * BY, BZZ = FB3B * BZ;
    double CXX = FB3C * CX, CYY = FB3C * CY, CZZ = FB3C * CZ;
    st->hx[I] = st->hx[I] - AXX - BXX;
    st->hy[I] = st->hy[I] - AYY - BYY;
    st->hz[I] = st->hz[I] - AZZ - BZZ;
    st->hx[J] = st->hx[J] + AXX - CXX;
    st->hy[J] = st->hy[J] + AYY - CYY;
    st->hz[J] = st->hz[J] + AZZ - CZZ;
    st->hx[K] = st->hx[K] + BXX + CXX;
    st->hy[K] = st->hy[K] + BYY + CYY;
    st->hz[K] = st->hz[K] + BZZ + CZZ;
    double VIX = AX * AXX + BX * BXX + CX * CXX;
    double VIY = AY * AYY + BY * BYY + CY * CYY;
    double VIZ = AZ * AZZ + BZ * BZZ + CZ * CZZ;
    s->virb = s->virb + VIX + VIY + VIZ;
    s->virfx = s->virfx + VIX;
    s->virfy = s->virfy + VIY;
    s->virfz = s->virfz + VIZ;
  }
}

/* ---------------------------------------------------------------- SCLFRC */
static void sclfrc(ox_state *st, int nnn) {
  st->lscfl = 0;
  if (!st->p.lscft) return;
  double fct = nnn == 1 ? st->p.ftscl * st->p.ftimes : st->p.ftscl;
  double *ax = nnn == 1 ? st->hx : nnn == 2 ? st->gx : st->fx;
  double *ay = nnn == 1 ? st->hy : nnn == 2 ? st->gy : st->fy;
  double *az = nnn == 1 ? st->hz : nnn == 2 ? st->gz : st->fz;
  for (int I = 1; I <= st->nstot; ++I) {
    double f = ax[I] * ax[I] + ay[I] * ay[I] + az[I] * az[I];
    f = sqrt(f) * fct * st->massdi[I];
    if (f > 1.0) {
      if (f > 1.0e20) {
        ax[I] = 0.; ay[I] = 0.; az[I] = 0.;
      } else {
        ax[I] = ax[I] / f; ay[I] = ay[I] / f; az[I] = az[I] / f;
      }
      st->lscfl = 1;
    }
  }
}

/* ---------------------------------------------------------------- GETCOM */
int ox_getcom(ox_state *st) {
  int N = 0, I = 0;
  for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP) {
    int NSBEG = st->isadr[ITYP] + 1, NSEND = st->isadr[ITYP + 1];
    double SUMM = st->summas[ITYP];
    for (int J = 1; J <= st->nspec[ITYP]; ++J) {
      I = I + 1;
      st->X[I] = 0.; st->Y[I] = 0.; st->Z[I] = 0.;
      st->PX[I] = 0.; st->PY[I] = 0.; st->PZ[I] = 0.;
      for (int IS = NSBEG; IS <= NSEND; ++IS) {
        N = N + 1;
        st->X[I] = st->X[I] + st->mass[IS] * st->sx[N];
        st->Y[I] = st->Y[I] + st->mass[IS] * st->sy[N];
        st->Z[I] = st->Z[I] + st->mass[IS] * st->sz[N];
        st->PX[I] = st->PX[I] + st->vx[N];
        st->PY[I] = st->PY[I] + st->vy[N];
        st->PZ[I] = st->PZ[I] + st->vz[N];
      }
      st->X[I] = st->X[I] / SUMM;
      st->Y[I] = st->Y[I] / SUMM;
      st->Z[I] = st->Z[I] / SUMM;
    }
  }
  for (int n = 1; n <= st->nstot; ++n) {
    int M = st->nnum[n];
    st->wx[n] = st->sx[n] - st->X[M];
    st->wy[n] = st->sy[n] - st->Y[M];
    st->wz[n] = st->sz[n] - st->Z[M];
  }
  for (int i = 1; i <= st->nop; ++i) pbc(st, &st->X[i], &st->Y[i], &st->Z[i]);
  for (int n = 1; n <= st->nstot; ++n) {
    int M = st->nnum[n];
    st->sx[n] = st->wx[n] + st->X[M];
    st->sy[n] = st->wy[n] + st->Y[M];
    st->sz[n] = st->wz[n] + st->Z[M];
  }
  return MDX_OK;
}

/* ---------------------------------------------------------------- GETEMP */
static int getemp(ox_state *st) {
  mdx_thermo *th = &st->th;
  int nt = st->ntypes;
  double VIRKX = 0., VIRKY = 0., VIRKZ = 0., VSQ = 0.;
  double tempr[NT + 5];
  for (int i = 0; i < NT + 5; ++i) tempr[i] = 0.;
  for (int I = 1; I <= st->nstot; ++I) {
    int ITYP = st->itype[I];
    if (st->lmove[ITYP]) {
      double VVX = st->massdi[I] * (st->vx[I] * st->vx[I]);
      double VVY = st->massdi[I] * (st->vy[I] * st->vy[I]);
      double VVZ = st->massdi[I] * (st->vz[I] * st->vz[I]);
      double VSC = VVX + VVY + VVZ;
      VIRKX = VIRKX + VVX;
      VIRKY = VIRKY + VVY;
      VIRKZ = VIRKZ + VVZ;
      VSQ = VSQ + VSC;
      tempr[ITYP] = tempr[ITYP] + 0.5 * VSC;
    }
  }
  double TEMP = 0.5 * VSQ;
  int NTYP1 = nt + 1;
  tempr[NTYP1] = TEMP;
  tempr[NTYP1 + 1] = VIRKX;
  tempr[NTYP1 + 2] = VIRKY;
  tempr[NTYP1 + 3] = VIRKZ;
  for (int i = 1; i <= NTYP1 + 3; ++i) th->ekin[i - 1] = tempr[i];
  th->tke = th->ekin[NTYP1 - 1];
  th->virkx = th->ekin[NTYP1];
  th->virky = th->ekin[NTYP1 + 1];
  th->virkz = th->ekin[NTYP1 + 2];
  for (int i = 1; i <= NTYP1 + 3; ++i) th->tempr[i - 1] = tempr[i];
  for (int ITYP = 1; ITYP <= nt; ++ITYP)
    th->tempr[ITYP - 1] = th->ekin[ITYP - 1] * st->p.tfact[ITYP - 1];
  th->temp = th->tke * st->p.convet;
  if (st->p.chktf > 0.0 &&
      (th->temp > st->p.chktf * st->p.trtemp || th->temp <= st->p.trtemp / st->p.chktf)) {
    snprintf(st->msg, sizeof st->msg, "Temperature control stopped the program: T=%g", th->temp);
    return MDX_ERR_NAN;
  }
  return MDX_OK;
}

/* ---------------------------------------------------------------- INV3B3 */
/* util.f:89-125: inverse by cofactors, IER 1 for a near-singular matrix,
 * 2 for a singular one (inverse zero). */
static void inv3b3(const double *A, double *AI, double *DET, int *IER) {
  AI[1] = A[5] * A[9] - A[6] * A[8];
  AI[2] = A[3] * A[8] - A[2] * A[9];
  AI[3] = A[2] * A[6] - A[3] * A[5];
  AI[4] = A[6] * A[7] - A[4] * A[9];
  AI[5] = A[1] * A[9] - A[3] * A[7];
  AI[6] = A[3] * A[4] - A[1] * A[6];
  AI[7] = A[4] * A[8] - A[5] * A[7];
  AI[8] = A[2] * A[7] - A[1] * A[8];
  AI[9] = A[1] * A[5] - A[2] * A[4];
  *DET = A[1] * AI[1] + A[4] * AI[2] + A[7] * AI[3];
  double SPUR = A[1] + A[5] + A[9];
  *IER = 0;
  if (fabs(*DET) < 1.e-6 * fabs(SPUR * SPUR * SPUR)) *IER = 1;
  double R;
  if (fabs(*DET) > 0.0) {
    R = 1.0 / *DET;
  } else {
    R = 0.0;
    *IER = 2;
  }
  for (int k = 1; k <= 9; ++k) AI[k] = R * AI[k];
}

/* ---------------------------------------------------------------- GETKIN */
/* service.f:611-735 without GETROT (LMOL1/LMOL2).  SUMMD comes in per type
 * (SUMMAS/(AVSNO*1000*UNITM*NBEADS)); MASSD(IS) is taken as 1/MASSDI of the
 * atom (within an ulp of the stored site mass); WX.. are the site vectors
 * GETCOM left.  out: EKTR, EKROT, EKINT, TKE, TTR, TROT, TINT. */
int ox_getkin(ox_state *st, const double *summd, double enerf_tempf, double fnop,
              double fnstr, double fnsti, double *out) {
  int N = 0;
  double EKTR = 0., EKROT = 0., TKE = 0.;
  for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP) {
    double SUMMD = summd[ITYP - 1];
    int NSS = st->nsits[ITYP];
    int ISB = st->isadr[ITYP] + 1, ISE = st->isadr[ITYP + 1];
    for (int J = 1; J <= st->nspec[ITYP]; ++J) {
      double PXJ = 0., PYJ = 0., PZJ = 0.;
      double TOR[10], TORI[10], DET;
      int IER;
      for (int k = 1; k <= 9; ++k) TOR[k] = 0.;
      for (int IS = ISB; IS <= ISE; ++IS) {
        N = N + 1;
        PXJ = PXJ + st->vx[N];
        PYJ = PYJ + st->vy[N];
        PZJ = PZJ + st->vz[N];
        TKE = TKE + 0.5 * (st->vx[N] * st->vx[N] + st->vy[N] * st->vy[N] +
                           st->vz[N] * st->vz[N]) * st->massdi[N];
        double MD = 1.0 / st->massdi[N];
        double WX = st->wx[N], WY = st->wy[N], WZ = st->wz[N];
        TOR[1] = TOR[1] + MD * (WY * WY + WZ * WZ);
        TOR[5] = TOR[5] + MD * (WX * WX + WZ * WZ);
        TOR[9] = TOR[9] + MD * (WX * WX + WY * WY);
        TOR[2] = TOR[2] - MD * WX * WY;
        TOR[3] = TOR[3] - MD * WX * WZ;
        TOR[6] = TOR[6] - MD * WY * WZ;
      }
      TOR[4] = TOR[2];
      TOR[7] = TOR[3];
      TOR[8] = TOR[6];
      inv3b3(TOR, TORI, &DET, &IER);
      EKTR = EKTR + 0.5 * (PXJ * PXJ + PYJ * PYJ + PZJ * PZJ) / SUMMD;
      double RXJ = 0., RYJ = 0., RZJ = 0.;
      N = N - NSS;
      for (int IS = ISB; IS <= ISE; ++IS) {
        N = N + 1;
        double FAC = st->mass[IS] / st->summas[ITYP];
        double VTX = st->vx[N] - PXJ * FAC;
        double VTY = st->vy[N] - PYJ * FAC;
        double VTZ = st->vz[N] - PZJ * FAC;
        RXJ = RXJ + (VTY * st->wz[N] - st->wy[N] * VTZ);
        RYJ = RYJ + (VTZ * st->wx[N] - st->wz[N] * VTX);
        RZJ = RZJ + (VTX * st->wy[N] - st->wx[N] * VTY);
      }
      double EROTM;
      if (IER == 0) {
        EROTM = 0.5 * (TORI[1] * RXJ * RXJ + (TORI[2] + TORI[4]) * RXJ * RYJ +
                       TORI[5] * RYJ * RYJ + (TORI[3] + TORI[7]) * RXJ * RZJ +
                       TORI[9] * RZJ * RZJ + (TORI[6] + TORI[8]) * RYJ * RZJ);
      } else {
        double ROTM = 0.;
        double PP = RXJ * RXJ + RYJ * RYJ + RZJ * RZJ;
        if (PP < 1.e-50) continue; /* go to 100 */
        N = N - NSS;
        for (int IS = ISB; IS <= ISE; ++IS) {
          N = N + 1;
          double SS = st->wx[N] * st->wx[N] + st->wy[N] * st->wy[N] + st->wz[N] * st->wz[N];
          double SP = st->wx[N] * RXJ + st->wy[N] * RYJ + st->wz[N] * RZJ;
          ROTM = ROTM + (1.0 / st->massdi[N]) * (SS * PP - SP * SP);
        }
        EROTM = ROTM >= 1.e-50 ? 0.5 * PP * PP / ROTM : 0.0;
      }
      EKROT = EKROT + EROTM;
    }
  }
  double EKINT = TKE - EKTR - EKROT;
  double TTR = fnop > 1.1 ? EKTR * enerf_tempf / (fnop - 1.0) : EKTR * enerf_tempf / fnop;
  double TROT = fnstr > 0.01 ? 3. * EKROT * enerf_tempf / fnstr : st->th.temp;
  double TINT = fnsti > 0.01 ? 3.0 * EKINT * enerf_tempf / fnsti : 0.;
  out[0] = EKTR; out[1] = EKROT; out[2] = EKINT; out[3] = TKE;
  out[4] = TTR; out[5] = TROT; out[6] = TINT;
  return MDX_OK;
}

/* ---------------------------------------------------------------- CHKMOM */
/* service.f:1081-1125 (one rank): remove the total momentum, GETEMP; dv:
 * the removed DVX, DVY, DVZ. */
int ox_chkmom(ox_state *st, double sumasd, double *dv) {
  double PT[3] = {0., 0., 0.};
  for (int I = 1; I <= st->nstot; ++I) {
    PT[0] = PT[0] + st->vx[I];
    PT[1] = PT[1] + st->vy[I];
    PT[2] = PT[2] + st->vz[I];
  }
  double DVX = PT[0] / sumasd, DVY = PT[1] / sumasd, DVZ = PT[2] / sumasd;
  for (int I = 1; I <= st->nstot; ++I) {
    st->vx[I] = st->vx[I] - DVX / st->massdi[I];
    st->vy[I] = st->vy[I] - DVY / st->massdi[I];
    st->vz[I] = st->vz[I] - DVZ / st->massdi[I];
  }
  getemp(st);
  if (dv) {
    dv[0] = DVX; dv[1] = DVY; dv[2] = DVZ;
  }
  return MDX_OK;
}

/* ------------------------------------------------------- force collectors */
int ox_fforces(ox_state *st, int laver, mdx_scalars *out) {
  (void)laver; /* CM_ADDF only adds to averaging accumulators (L5) */
  zerofs(st, 1);
  localf(st);
  getbnd(st);
  getang(st);
  gettrs(st);
  sclfrc(st, 1);
  st->s.mbsh = st->mbsh;
  st->s.mbln = st->mbln;
  st->s.lscfl = st->lscfl;
  if (out) *out = st->s;
  return MDX_OK;
}

static void cm_addl_wirs(ox_state *st) {
  for (int N = 1; N <= st->nstot; ++N) {
    int M = st->nnum[N];
    st->s.wirs = st->s.wirs - st->gx[N] * (st->sx[N] - st->X[M]) -
                 st->gy[N] * (st->sy[N] - st->Y[M]) -
                 st->gz[N] * (st->sz[N] - st->Z[M]);
  }
}

int ox_set_pullback(ox_state *st, const mdx_pullback *pb) {
  free(st->pull_atom);
  free(st->pull_ref);
  st->pull_atom = NULL;
  st->pull_ref = NULL;
  st->pull_on = 0;
  if (!pb) return MDX_OK;
  st->pb = *pb;
  st->pull_nstep = pb->nstep;
  if (pb->npull > 0) {
    st->pull_atom = (int *)xcalloc((size_t)pb->npull + 1, sizeof(int));
    st->pull_ref = (double *)xcalloc(3 * (size_t)pb->npull + 3, sizeof(double));
    for (int k = 0; k < pb->npull; ++k) {
      st->pull_atom[k + 1] = pb->inpl[k];
      st->pull_ref[3 * k + 0] = pb->xpl[k];
      st->pull_ref[3 * k + 1] = pb->ypl[k];
      st->pull_ref[3 * k + 2] = pb->zpl[k];
    }
  }
  st->pull_on = pb->ldrag || pb->npull > 0 || pb->iext == 1;
  return MDX_OK;
}

/* PULLBACK, forces.f:1756-1799 */
static void pullback(ox_state *st) {
  if (!st->pull_on) return;
  const mdx_pullback *pb = &st->pb;
  if (pb->ldrag)
    for (int I = 1; I <= st->nstot; ++I) {
      int ITYP = st->itype[I];
      if (pb->ldragt[ITYP - 1]) {
        int IS = st->nsite[I];
        (void)IS;
        st->gz[I] = st->gz[I] + (1.0 / st->massdi[I]) * pb->fdrag[ITYP - 1];
      }
    }
  if (pb->npull > 0)
    for (int IL = 1; IL <= pb->npull; ++IL) {
      int I = st->pull_atom[IL];
      double DX = st->sx[I] - st->pull_ref[3 * (IL - 1) + 0];
      double DY = st->sy[I] - st->pull_ref[3 * (IL - 1) + 1];
      double DZ = st->sz[I] - st->pull_ref[3 * (IL - 1) + 2];
      st->gx[I] = st->gx[I] - pb->rlr * DX;
      st->gy[I] = st->gy[I] - pb->rlr * DY;
      st->gz[I] = st->gz[I] - pb->rlr * DZ;
    }
  if (pb->iext == 1) {
    double FULTIM = pb->tim + st->pull_nstep * pb->dt;
    double EFIELD = pb->exampl * cos(pb->exfreq * FULTIM * 0.5 / PI);
    for (int I = 1; I <= st->nstot; ++I) st->gz[I] = st->gz[I] + st->q[I] * EFIELD;
  }
}

int ox_slforces(ox_state *st, mdx_scalars *out) {
  int rc;
  zerofs(st, 2);
  st->s.qpe = 0.;
  if ((rc = furir(st))) return rc;
  eterms(st);
  forces_long(st);
  cm_addl_wirs(st); /* CM_ADDLF, scalar.f:77-82 */
  pullback(st);
  sclfrc(st, 2);
  st->s.mbsh = st->mbsh;
  st->s.mbln = st->mbln;
  st->s.lscfl = st->lscfl;
  if (out) *out = st->s;
  return MDX_OK;
}

int ox_allforce(ox_state *st, mdx_scalars *out) {
  int rc;
  zerofs(st, 1);
  zerofs(st, 2);
  st->s.qpe = 0.;
  localf(st);
  getbnd(st);
  getang(st);
  gettrs(st);
  if ((rc = furir(st))) return rc;
  eterms(st);
  forces_long(st);
  for (int N = 1; N <= st->nstot; ++N) { /* CM_ADDLA, scalar.f:106-113 */
    st->fx[N] = st->gx[N] + st->hx[N];
    st->fy[N] = st->gy[N] + st->hy[N];
    st->fz[N] = st->gz[N] + st->hz[N];
    int M = st->nnum[N];
    st->s.wirs = st->s.wirs - st->gx[N] * (st->sx[N] - st->X[M]) -
                 st->gy[N] * (st->sy[N] - st->Y[M]) -
                 st->gz[N] * (st->sz[N] - st->Z[M]);
  }
  pullback(st); /* into G after F = G + H, as ALLFORCE orders it */
  sclfrc(st, 3);
  st->s.mbsh = st->mbsh;
  st->s.mbln = st->mbln;
  st->s.lscfl = st->lscfl;
  if (out) *out = st->s;
  return MDX_OK;
}

/* ---------------------------------------------------------------- SCALING */
static void scale_v(ox_state *st, double sx_, double sy_, double sz_) {
  for (int I = 1; I <= st->nstot; ++I)
    if (st->lmove[st->itype[I]]) {
      st->vx[I] = st->vx[I] * sx_;
      st->vy[I] = st->vy[I] * sy_;
      st->vz[I] = st->vz[I] * sz_;
    }
}

static void scale_v_types(ox_state *st, double h) {
  for (int I = 1; I <= st->nstot; ++I) {
    int ITYP = st->itype[I];
    double SCV = 1. - st->th.scm[ITYP - 1] * h;
    if (st->lmove[ITYP]) {
      st->vx[I] = st->vx[I] * SCV;
      st->vy[I] = st->vy[I] * SCV;
      st->vz[I] = st->vz[I] * SCV;
    }
  }
}

static int npt_guard(ox_state *st, double f) {
  if (fabs(f) >= 0.1) {
    st->th.npt_fail += 1;
    if (st->th.npt_fail > 100) {
      snprintf(st->msg, sizeof st->msg, "repeated failure of NPT-algorithm");
      return MDX_ERR_NAN;
    }
  }
  return MDX_OK;
}

static int scaling(ox_state *st, int IAL) {
  mdx_thermo *th = &st->th;
  const mdx_params *p = &st->p;
  mdx_scalars *s = &st->s;
  int rc;
  double DPE[5], DTE[NT + 1];
  const double TSTEP = p->tstep, HTSTEP = 0.5 * p->tstep;
  const double FNST = p->fnst;
  if (IAL == 3 && p->lnvt) {
    if (p->lsctd) {
      scale_v_types(st, TSTEP);
    } else {
      double SCV = 1. - th->sc * TSTEP;
      scale_v(st, SCV, SCV, SCV);
    }
  }
  if ((rc = getemp(st))) return rc;
  double VIRSUM = s->vir1 + s->vir2 + s->virb + s->pels1 + s->pels2 + s->spe + p->vird +
                  th->vira[0] + th->vira[1] + th->vira[2];
  double WIRSUM = s->vir1 + s->vir2 + s->pels1 + s->pels2 + s->spe + p->vird + s->wirs + s->wirss;
  double VOL = st->vol;
  double TRIDEE = p->tridee_coef / VOL;
  double TRID = 2. * th->tke * p->unitp / (3. * VOL) - TRIDEE;
  double TRIDM = p->tridm_coef * th->temp / VOL - TRIDEE;
  double TRIDX = th->virkx * p->unitp / VOL - TRIDEE / 3.;
  double TRIDY = th->virky * p->unitp / VOL - TRIDEE / 3.;
  double TRIDZ = th->virkz * p->unitp / VOL - TRIDEE / 3.;
  th->tryck = VIRSUM * p->unitp / (3. * VOL) + TRID;
  th->tryckm = WIRSUM * p->unitp / (3. * VOL) + TRIDM;
  th->tryckx = (s->virx + s->virfx + p->vird / 3. + th->vira[0]) * p->unitp / VOL + TRIDX;
  th->trycky = (s->viry + s->virfy + p->vird / 3. + th->vira[1]) * p->unitp / VOL + TRIDY;
  th->tryckz = (s->virz + s->virfz + p->vird / 3. + th->vira[2]) * p->unitp / VOL + TRIDZ;
  double DKE = th->temp / p->trtemp - 1.0;
  for (int I = 1; I <= st->ntypes; ++I) DTE[I] = th->tempr[I - 1] / p->trtemp - 1.0;
  if (st->lscfl) {
    for (int I = 1; I <= 4; ++I) DPE[I] = 0.;
  } else {
    DPE[1] = p->lshejk ? th->tryckm - p->trpres : th->tryck - p->trpres;
    DPE[2] = th->tryckx - p->trpresx;
    DPE[3] = th->trycky - p->trpresy;
    if (p->lp_xy) {
      DPE[2] = 0.5 * (DPE[2] + DPE[3]);
      DPE[3] = DPE[2];
    }
    DPE[4] = th->tryckz - p->trpresz;
  }
  const double DQT = p->dqt, DQP = p->dqp, RTP = p->rtp;
  if (IAL == 1) {
    if (p->lnvt) {
      if (p->lsctd) {
        double SCA = 0.;
        for (int I = 1; I <= st->ntypes; ++I) {
          th->scm[I - 1] = th->scm[I - 1] + DTE[I] * DQT * HTSTEP;
          SCA = SCA + th->scm[I - 1] * th->ekin[I - 1];
        }
        th->sc = SCA / th->tke;
      } else {
        th->sc = th->sc + DKE * DQT * HTSTEP;
      }
      if (p->lnpt) {
        if (p->lsctd) {
          double SCA = 0.;
          for (int I = 1; I <= st->ntypes; ++I) {
            th->scm[I - 1] = th->scm[I - 1] + (th->scl * th->scl * RTP - DQT / FNST) * HTSTEP;
            SCA = SCA + th->scm[I - 1] * th->ekin[I - 1];
          }
          th->sc = SCA / th->tke;
        } else {
          th->sc = th->sc + (th->scl * th->scl * RTP - DQT / FNST) * HTSTEP;
        }
        if (p->lsep) {
          th->sclx = th->sclx + DQP * (VOL * DPE[2] + 2. * th->tke / FNST - th->sclx * th->sc) * HTSTEP;
          th->scly = th->scly + DQP * (VOL * DPE[3] + 2. * th->tke / FNST - th->scly * th->sc) * HTSTEP;
          if (p->lp_xy) {
            th->sclx = 0.5 * (th->sclx + th->scly);
            th->scly = th->sclx;
          }
          th->sclz = th->sclz + DQP * (VOL * DPE[4] + 2. * th->tke / FNST - th->sclz * th->sc) * HTSTEP;
          th->scl = th->sclx + th->scly + th->sclz;
        } else {
          th->scl = th->scl + DQP * (3. * VOL * DPE[1] + 6. * th->tke / FNST - th->scl * th->sc) * HTSTEP;
          th->sclx = th->scl;
          th->scly = th->scl;
          th->sclz = th->scl;
          if ((rc = npt_guard(st, th->scl * HTSTEP))) return rc;
        }
        double SCVX = 1. - ((1. - 3. / FNST) * th->sclx + th->sc) * HTSTEP;
        double SCVY = 1. - ((1. - 3. / FNST) * th->scly + th->sc) * HTSTEP;
        double SCVZ = 1. - ((1. - 3. / FNST) * th->sclz + th->sc) * HTSTEP;
        if (p->lp_xy) {
          SCVX = 0.5 * (SCVX + SCVY);
          SCVY = SCVX;
        }
        double DRCX = TSTEP * th->sclx, DRCY = TSTEP * th->scly, DRCZ = TSTEP * th->sclz;
        double DRC = (DRCX + DRCY + DRCZ) / 3.;
        double DRCV = DRC * HTSTEP;
        DRCX = 1. + DRCX + 0.5 * (DRCX * DRCX);
        DRCY = 1. + DRCY + 0.5 * (DRCY * DRCY);
        DRCZ = 1. + DRCZ + 0.5 * (DRCZ * DRCZ);
        for (int I = 1; I <= st->nstot; ++I) {
          if (st->lmove[st->itype[I]]) {
            st->vx[I] = st->vx[I] * SCVX;
            st->vy[I] = st->vy[I] * SCVY;
            st->vz[I] = st->vz[I] * SCVZ;
            st->sx[I] = st->sx[I] * DRCX + st->vx[I] * DRCV * st->massdi[I];
            st->sy[I] = st->sy[I] * DRCY + st->vy[I] * DRCV * st->massdi[I];
            st->sz[I] = st->sz[I] * DRCZ + st->vz[I] * DRCV * st->massdi[I];
          }
        }
        reclen(st, DRCX, DRCY, DRCZ);
      } else {
        if ((rc = getemp(st))) return rc;
        if (p->lsctd) {
          scale_v_types(st, HTSTEP);
        } else {
          double SCV = 1. - th->sc * HTSTEP;
          scale_v(st, SCV, SCV, SCV);
        }
      }
      th->eabs = th->eabs - (th->sc + th->scl * (1. - 3. / FNST)) * th->tke * TSTEP;
    }
  } else if (IAL == 2) {
    if (p->lnvt) {
      if (p->lsctd) {
        scale_v_types(st, HTSTEP);
      } else {
        double SCV = 1. - th->sc * HTSTEP;
        scale_v(st, SCV, SCV, SCV);
      }
      if (p->lnpt) {
        double SCVX = 1. - (1. - 3. / p->fnop) * th->sclx * HTSTEP;
        double SCVY = 1. - (1. - 3. / p->fnop) * th->scly * HTSTEP;
        double SCVZ = 1. - (1. - 3. / p->fnop) * th->sclz * HTSTEP;
        if (p->lp_xy) {
          SCVX = 0.5 * (SCVX + SCVY);
          SCVY = SCVX;
        }
        scale_v(st, SCVX, SCVY, SCVZ);
        if ((rc = getemp(st))) return rc;
        if (p->lsep) {
          th->sclx = th->sclx + DQP * (VOL * DPE[2] + 2. * th->tke / FNST - th->sclx * th->sc) * HTSTEP;
          th->scly = th->scly + DQP * (VOL * DPE[3] + 2. * th->tke / FNST - th->scly * th->sc) * HTSTEP;
          if (p->lp_xy) {
            th->sclx = 0.5 * (th->sclx + th->scly);
            th->scly = th->sclx;
          }
          th->sclz = th->sclz + DQP * (VOL * DPE[4] + 2. * th->tke / FNST - th->sclz * th->sc) * HTSTEP;
          th->scl = th->sclx + th->scly + th->sclz;
        } else {
          th->scl = th->scl + DQP * (3. * VOL * DPE[1] + 6. * th->tke / FNST - th->scl * th->sc) * HTSTEP;
          th->sclx = th->scl;
          th->scly = th->scl;
          th->sclz = th->scl;
          if ((rc = npt_guard(st, th->scl * HTSTEP))) return rc;
        }
        th->sc = th->sc + (th->scl * th->scl * RTP - DQT / FNST) * HTSTEP;
        if (p->lsctd)
          for (int I = 1; I <= st->ntypes; ++I)
            th->scm[I - 1] = th->scm[I - 1] + (th->scl * th->scl * RTP - DQT / FNST) * HTSTEP;
      } else {
        if ((rc = getemp(st))) return rc;
      }
      if (p->lsctd) {
        double SCA = 0.;
        for (int I = 1; I <= st->ntypes; ++I) {
          DTE[I] = th->tempr[I - 1] / p->trtemp - 1.0;
          th->scm[I - 1] = th->scm[I - 1] + DTE[I] * DQT * HTSTEP;
          SCA = SCA + th->scm[I - 1] * th->ekin[I - 1];
        }
        th->sc = SCA / th->tke;
      } else {
        DKE = th->temp / p->trtemp - 1.0;
        th->sc = th->sc + DKE * DQT * HTSTEP;
      }
      th->eabs = th->eabs - (th->sc + th->scl * (1. - 3. / FNST)) * th->tke * TSTEP;
    }
  } else if (IAL == 3) {
    if (p->lnvt) {
      th->sc = th->sc + DKE * DQT * TSTEP;
      if (p->lsctd) {
        double SCA = 0.;
        for (int I = 1; I <= st->ntypes; ++I) {
          th->scm[I - 1] = th->scm[I - 1] + DTE[I] * DQT * TSTEP;
          SCA = SCA + th->scm[I - 1] * th->ekin[I - 1];
        }
        th->sc = SCA / th->tke;
      }
      if (p->lnpt) {
        if (p->lsep) {
          th->sclx = th->sclx + DQP * (VOL * DPE[2] + 2. * th->tke / FNST - th->sclx * th->sc) * TSTEP;
          th->scly = th->scly + DQP * (VOL * DPE[3] + 2. * th->tke / FNST - th->scly * th->sc) * TSTEP;
          if (p->lp_xy) {
            th->sclx = 0.5 * (th->sclx + th->scly);
            th->scly = th->sclx;
          }
          th->sclz = th->sclz + DQP * (VOL * DPE[4] + 2. * th->tke / FNST - th->sclz * th->sc) * TSTEP;
          th->scl = th->sclx + th->scly + th->sclz;
        } else {
          th->scl = th->scl + DQP * (3. * VOL * DPE[1] + 6. * th->tke / FNST - th->scl * th->sc) * TSTEP;
          th->sclx = th->scl;
          th->scly = th->scl;
          th->sclz = th->scl;
          if ((rc = npt_guard(st, th->scl * TSTEP))) return rc;
        }
        double SCV = ((1. - 3. / FNST) * th->scl) * TSTEP;
        double DRCX = TSTEP * th->sclx, DRCY = TSTEP * th->scly, DRCZ = TSTEP * th->sclz;
        for (int IMOL = 1; IMOL <= st->nop; ++IMOL) {
          int ITYP = st->itm[IMOL];
          double SUMM = st->summas[ITYP];
          if (!st->lmove[ITYP]) continue;
          double XC = 0., YC = 0., ZC = 0., PXC = 0., PYC = 0., PZC = 0.;
          int IBEG = st->isaddr[ITYP] + 1 + st->nsits[ITYP] * (IMOL - st->iaddr[ITYP] - 1);
          int IEND = st->isaddr[ITYP] + st->nsits[ITYP] * (IMOL - st->iaddr[ITYP]);
          for (int I = IBEG; I <= IEND; ++I) {
            int IS = st->nsite[I];
            XC = XC + st->mass[IS] * st->sx[I];
            YC = YC + st->mass[IS] * st->sy[I];
            ZC = ZC + st->mass[IS] * st->sz[I];
            PXC = PXC + st->vx[I];
            PYC = PYC + st->vy[I];
            PZC = PZC + st->vz[I];
          }
          XC = XC / SUMM;
          YC = YC / SUMM;
          ZC = ZC / SUMM;
          double DVX = PXC * SCV, DVY = PYC * SCV, DVZ = PZC * SCV;
          double DXC = XC * DRCX, DYC = YC * DRCY, DZC = ZC * DRCZ;
          for (int I = IBEG; I <= IEND; ++I) {
            int IS = st->nsite[I];
            double FAC = st->mass[IS] / SUMM;
            st->vx[I] = st->vx[I] - DVX * FAC;
            st->vy[I] = st->vy[I] - DVY * FAC;
            st->vz[I] = st->vz[I] - DVZ * FAC;
            st->sx[I] = st->sx[I] + DXC;
            st->sy[I] = st->sy[I] + DYC;
            st->sz[I] = st->sz[I] + DZC;
          }
        }
        DRCX = DRCX + 1.;
        DRCY = DRCY + 1.;
        DRCZ = DRCZ + 1.;
        reclen(st, DRCX, DRCY, DRCZ);
        th->sc = th->sc + (th->scl * th->scl * RTP - DQT / FNST) * TSTEP;
        if (p->lsctd) {
          double SCA = 0.;
          for (int I = 1; I <= st->ntypes; ++I) {
            th->scm[I - 1] = th->scm[I - 1] + (th->scl * th->scl * RTP - DQT / FNST) * TSTEP;
            SCA = SCA + th->scm[I - 1] * th->ekin[I - 1];
          }
          th->sc = SCA / th->tke;
        }
      }
      th->eabs = th->eabs - (th->sc + th->scl * (1. - 3. / FNST)) * th->tke * TSTEP;
    }
  }
  if (p->lsclt && (IAL == 2 || IAL == 3)) {
    if (p->lsctd) {
      for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP) {
        if (fabs(p->trtemp - th->tempr[ITYP - 1]) > p->tdelt && st->lmove[ITYP]) {
          double SCV = sqrt(p->trtemp / th->tempr[ITYP - 1]);
          for (int I = st->isaddr[ITYP] + 1; I <= st->isaddr[ITYP + 1]; ++I) {
            st->vx[I] = SCV * st->vx[I];
            st->vy[I] = SCV * st->vy[I];
            st->vz[I] = SCV * st->vz[I];
          }
          th->nscale += 1;
        }
      }
    } else if (fabs(p->trtemp - th->temp) > p->tdelt) {
      double SCV = sqrt(p->trtemp / th->temp);
      scale_v(st, SCV, SCV, SCV);
      th->nscale += 1;
    }
    if ((rc = getemp(st))) return rc;
  }
  return MDX_OK;
}

/* ----------------------------------------------------------------- SHEJK */
static void shejk(ox_state *st, int IMOL, unsigned char *moving,
                  unsigned char *moved) {
  mdx_thermo *th = &st->th;
  int ITYP = st->itm[IMOL];
  int NRBS = st->nrb[ITYP];
  if (st->ishejk[ITYP] <= 0 || NRBS <= 0) return;
  const int MAXIT = st->p.maxit > 0 ? st->p.maxit : 2000;
  double TOL2 = st->p.toler * st->p.toler;
  double TSTEP = st->p.tstep;
  int NBBEG = st->iadb[ITYP];
  int NBEND = NBBEG + NRBS - 1;
  int ISHF = st->isaddr[ITYP] + st->nsits[ITYP] * (IMOL - st->iaddr[ITYP] - 1);
  int ISBEG = ISHF + 1, ISEND = ISHF + st->nsits[ITYP];
  for (int I = ISBEG; I <= ISEND; ++I) {
    st->fx[I] = st->sx[I];
    st->fy[I] = st->sy[I];
    st->fz[I] = st->sz[I];
  }
  for (int M = NBBEG; M <= NBEND; ++M)
    if (st->lcon[M]) {
      int LI = st->ib[M] + ISHF, LJ = st->jb[M] + ISHF;
      moving[LI] = 0; moved[LI] = 1;
      moving[LJ] = 0; moved[LJ] = 1;
    }
  int ITER = 0, DONE = 0;
  for (;;) {
    if (ITER > MAXIT) break;
    if (DONE) break;
    DONE = 1;
    for (int M = NBBEG; M <= NBEND; ++M) {
      if (!st->lcon[M]) continue;
      int I = st->ib[M] + ISHF, J = st->jb[M] + ISHF;
      if (!(moved[I] || moved[J])) continue;
      double BNDSQ = st->rb[M] * st->rb[M];
      double BXN = st->sx[I] - st->sx[J];
      double BYN = st->sy[I] - st->sy[J];
      double BZN = st->sz[I] - st->sz[J];
      pbc(st, &BXN, &BYN, &BZN);
      double BSQ = BXN * BXN + BYN * BYN + BZN * BZN;
      double DIFFSQ = BNDSQ - BSQ;
      if (fabs(DIFFSQ) > (BNDSQ * TOL2)) {
        double DXN = st->ox[I] - st->ox[J];
        double DYN = st->oy[I] - st->oy[J];
        double DZN = st->oz[I] - st->oz[J];
        pbc(st, &DXN, &DYN, &DZN);
        double VDOT = BXN * DXN + BYN * DYN + BZN * DZN;
        double RMA = st->massdi[I], RMB = st->massdi[J];
        double GAB = DIFFSQ / (2.0 * (RMA + RMB) * VDOT);
        DXN = DXN * GAB;
        DYN = DYN * GAB;
        DZN = DZN * GAB;
        st->sx[I] = st->sx[I] + RMA * DXN;
        st->sy[I] = st->sy[I] + RMA * DYN;
        st->sz[I] = st->sz[I] + RMA * DZN;
        st->sx[J] = st->sx[J] - RMB * DXN;
        st->sy[J] = st->sy[J] - RMB * DYN;
        st->sz[J] = st->sz[J] - RMB * DZN;
        moving[I] = 1;
        moving[J] = 1;
        DONE = 0;
      }
    }
    for (int M = NBBEG; M <= NBEND; ++M)
      if (st->lcon[M]) {
        moved[st->ib[M] + ISHF] = 0;
        moved[st->jb[M] + ISHF] = 0;
      }
    for (int M = NBBEG; M <= NBEND; ++M)
      if (st->lcon[M]) {
        int I = st->ib[M] + ISHF, J = st->jb[M] + ISHF;
        if (moving[I]) moved[I] = 1;
        if (moving[J]) moved[J] = 1;
        moving[I] = 0;
        moving[J] = 0;
      }
    ITER = ITER + 1;
  }
  if (ITER > th->shake_iter_max) th->shake_iter_max = ITER;
  if (ITER >= MAXIT) th->shake_fail += 1;
  for (int I = ISBEG; I <= ISEND; ++I) {
    double DIX = (st->sx[I] - st->fx[I]) / (st->massdi[I] * TSTEP);
    double DIY = (st->sy[I] - st->fy[I]) / (st->massdi[I] * TSTEP);
    double DIZ = (st->sz[I] - st->fz[I]) / (st->massdi[I] * TSTEP);
    th->viran[0] = th->viran[0] + DIX * st->ox[I] / TSTEP;
    th->viran[1] = th->viran[1] + DIY * st->oy[I] / TSTEP;
    th->viran[2] = th->viran[2] + DIZ * st->oz[I] / TSTEP;
    st->vx[I] = st->vx[I] + DIX;
    st->vy[I] = st->vy[I] + DIY;
    st->vz[I] = st->vz[I] + DIZ;
  }
}

static void fill_record(ox_state *st, int mstep, mdx_step_record *r) {
  mdx_scalars *s = &st->s;
  mdx_thermo *th = &st->th;
  memset(r, 0, sizeof *r);
  r->mstep = mstep;
  r->mbsh = st->mbsh;
  r->mbln = st->mbln;
  r->shake_iter = th->shake_iter_max;
  r->pe1 = s->pe1; r->pels1 = s->pels1; r->pe2 = s->pe2; r->pels2 = s->pels2;
  r->spe = s->spe; r->pint = s->pint;
  r->vir1 = s->vir1; r->vir2 = s->vir2; r->virb = s->virb;
  r->virx = s->virx; r->viry = s->viry; r->virz = s->virz;
  r->virfx = s->virfx; r->virfy = s->virfy; r->virfz = s->virfz;
  r->wirs = s->wirs; r->wirss = s->wirss;
  r->tke = th->tke; r->temp = th->temp; r->sc = th->sc; r->scl = th->scl;
  r->tryck = th->tryck; r->tryckm = th->tryckm;
  r->boxl = st->boxl; r->boyl = st->boyl; r->bozl = st->bozl; r->vol = st->vol;
  r->eabs = th->eabs;
}

/* ---------------------------------------------------------------- DOUBLE */
static void kick(ox_state *st, const double *ax, const double *ay,
                 const double *az, double h) {
  for (int I = 1; I <= st->nstot; ++I)
    if (st->lmove[st->itype[I]]) {
      st->vx[I] = st->vx[I] + h * ax[I];
      st->vy[I] = st->vy[I] + h * ay[I];
      st->vz[I] = st->vz[I] + h * az[I];
    }
}

int ox_double_steps(ox_state *st, int32_t nsteps, int32_t mstep0,
                    mdx_step_record *rec) {
  int rc;
  const int NFREQ = st->p.nfreq;
  const int NFREQ2 = NFREQ / 2 + 1;
  const double HTSTEP = 0.5 * st->p.tstep;
  const double TSTEB = st->p.tsteb, HTSTEB = 0.5 * st->p.tsteb;
  for (int NSTEP = 1; NSTEP <= nsteps; ++NSTEP) {
    int MSTEP = mstep0 + NSTEP;
    st->pull_nstep++;
    if ((rc = scaling(st, 1))) return rc;
    kick(st, st->gx, st->gy, st->gz, HTSTEP);
    int LMEM = 0;
    for (int NSTEB = 1; NSTEB <= NFREQ; ++NSTEB) {
      for (int I = 1; I <= st->nstot; ++I)
        if (st->lmove[st->itype[I]]) {
          st->vx[I] = st->vx[I] + HTSTEB * st->hx[I];
          st->vy[I] = st->vy[I] + HTSTEB * st->hy[I];
          st->vz[I] = st->vz[I] + HTSTEB * st->hz[I];
          st->sx[I] = st->vx[I] * TSTEB * st->massdi[I] + st->sx[I];
          st->sy[I] = st->vy[I] * TSTEB * st->massdi[I] + st->sy[I];
          st->sz[I] = st->vz[I] * TSTEB * st->massdi[I] + st->sz[I];
        }
      ox_getcom(st);
      if (NSTEB == NFREQ2 && list_due(st, MSTEP))
        if ((rc = ox_chcnb(st, NULL, NULL))) return rc;
      if (NSTEB == NFREQ) {
        if ((rc = ox_slforces(st, NULL))) return rc;
        LMEM = st->lscfl;
        ox_fforces(st, 1, NULL);
      } else {
        ox_fforces(st, 0, NULL);
      }
      kick(st, st->hx, st->hy, st->hz, HTSTEB);
    }
    if (LMEM) st->lscfl = 1;
    kick(st, st->gx, st->gy, st->gz, HTSTEP);
    if ((rc = scaling(st, 2))) return rc;
    if (rec) fill_record(st, MSTEP, &rec[NSTEP - 1]);
  }
  return MDX_OK;
}

int ox_double(ox_state *st, int32_t nsteps, int32_t nsttot,
              mdx_step_record *rec) {
  int rc;
  st->th.vira[0] = st->th.vira[1] = st->th.vira[2] = 0.;
  if ((rc = ox_chcnb(st, NULL, NULL))) return rc;
  ox_getcom(st);
  if ((rc = ox_slforces(st, NULL))) return rc;
  ox_fforces(st, 1, NULL);
  return ox_double_steps(st, nsteps, nsttot, rec);
}

/* ---------------------------------------------------------------- SULTAN */
int ox_sultan_steps(ox_state *st, int32_t nsteps, int32_t mstep0,
                    mdx_step_record *rec) {
  int rc;
  const double TSTEP = st->p.tstep;
  unsigned char *moving = (unsigned char *)xcalloc((size_t)st->nstot + 1, 1);
  unsigned char *moved = (unsigned char *)xcalloc((size_t)st->nstot + 1, 1);
  for (int NSTEP = 1; NSTEP <= nsteps; ++NSTEP) {
    int MSTEP = mstep0 + NSTEP;
    st->pull_nstep++;
    for (int I = 1; I <= st->nstot; ++I)
      if (st->lmove[st->itype[I]]) {
        st->ox[I] = st->sx[I];
        st->oy[I] = st->sy[I];
        st->oz[I] = st->sz[I];
      }
    for (int I = 1; I <= st->nstot; ++I)
      if (st->lmove[st->itype[I]]) {
        st->vx[I] = st->vx[I] + TSTEP * st->fx[I];
        st->vy[I] = st->vy[I] + TSTEP * st->fy[I];
        st->vz[I] = st->vz[I] + TSTEP * st->fz[I];
        st->sx[I] = st->sx[I] + TSTEP * st->vx[I] * st->massdi[I];
        st->sy[I] = st->sy[I] + TSTEP * st->vy[I] * st->massdi[I];
        st->sz[I] = st->sz[I] + TSTEP * st->vz[I] * st->massdi[I];
      }
    st->th.viran[0] = st->th.viran[1] = st->th.viran[2] = 0.;
    st->th.shake_iter_max = 0;
    if (st->p.lshejk)
      for (int IMOL = 1; IMOL <= st->nop; ++IMOL)
        if (st->lmove[st->itm[IMOL]]) shejk(st, IMOL, moving, moved);
    if (MSTEP == 1) {
      if ((rc = getemp(st))) goto out;
      double FTMP = sqrt(st->p.trtemp / st->th.temp);
      for (int N = 1; N <= st->nstot; ++N) {
        st->vx[N] = st->vx[N] * FTMP;
        st->vy[N] = st->vy[N] * FTMP;
        st->vz[N] = st->vz[N] * FTMP;
      }
    }
    for (int k = 0; k < 3; ++k) st->th.vira[k] = st->th.viran[k];
    if ((rc = scaling(st, 3))) goto out;
    ox_getcom(st);
    if (list_due(st, MSTEP))
      if ((rc = ox_chcnb(st, NULL, NULL))) goto out;
    if ((rc = ox_allforce(st, NULL))) goto out;
    if (rec) fill_record(st, MSTEP, &rec[NSTEP - 1]);
  }
  rc = MDX_OK;
out:
  free(moving);
  free(moved);
  return rc;
}

int ox_sultan(ox_state *st, int32_t nsteps, int32_t nsttot,
              mdx_step_record *rec) {
  int rc;
  if ((rc = ox_chcnb(st, NULL, NULL))) return rc;
  if ((rc = getemp(st))) return rc;
  if ((rc = ox_allforce(st, NULL))) return rc;
  return ox_sultan_steps(st, nsteps, nsttot, rec);
}

/* --------------------------------------------------- DIFFUR / DIFEN */
/* Energy differences of an expanded-ensemble move from coupling ec_old
 * (EC(ME)) to ec_new (EC(ME1)): out = EFN, EFO (DIFFUR mdee.f:265-376) and
 * EEN, EEO (DIFEN mdee.f:379-536), on the current positions, charges and
 * lists.  The k-set is the last INIFUR's. */
static double ee_pair_energy(const ox_state *st, int ISP, int JSP, double EEALN1, double RSHO,
                             double RSHN, double *een) {
  int ITYP = st->itype[ISP], JTYP = st->itype[JSP];
  int ISB = st->nsite[ISP], JSB = st->nsite[JSP];
  int ISN = st->inbt[ISB], JSN = st->inbt[JSB];
  int nb = st->nnbt;
  double A6O = st->a6lj[IDX2(ISN, JSN, nb)], B12O = st->b12lj[IDX2(ISN, JSN, nb)];
  double QIJO = st->q[ISP] * st->q[JSP] * st->p.coulf;
  double ESCI = st->iee[ITYP] == 0 ? EEALN1 : 1.0;
  double ESCL = ESCI;
  if (st->iee[JTYP] == 0) {
    ESCL = ESCI * EEALN1;
    ESCI = EEALN1;
  }
  double A6N = ESCI * st->a6lj0[IDX2(ISN, JSN, nb)];
  double B12N = ESCI * st->b12lj0[IDX2(ISN, JSN, nb)];
  double QIJN = ESCL * st->charge[ISB] * st->charge[JSB] * st->p.coulf;
  double DX = st->sx[ISP] - st->sx[JSP];
  double DY = st->sy[ISP] - st->sy[JSP];
  double DZ = st->sz[ISP] - st->sz[JSP];
  pbc(st, &DX, &DY, &DZ);
  double RR = DX * DX + DY * DY + DZ * DZ;
  double R1 = sqrt(RR);
  double R1O = R1 + RSHO, R1N = R1 + RSHN;
  double R1OI = 1. / R1O, R1NI = 1. / R1N;
  double ALPHAR = st->p.alphad * R1;
  double TTT = 1.0 / (1.0 + B1 * ALPHAR);
  double ERFCR = ((((A5 * TTT + A4) * TTT + A3) * TTT + A2) * TTT + A1) * TTT *
                 exp(-(ALPHAR * ALPHAR));
  double EESO = QIJO * ERFCR * R1OI, EESN = QIJN * ERFCR * R1NI;
  double R6IO = pow(R1OI, 6), R6IN = pow(R1NI, 6);
  double ESRO = (A6O + B12O * R6IO) * R6IO;
  double ESRN = (A6N + B12N * R6IN) * R6IN;
  *een += EESN + ESRN;
  return EESO + ESRO;
}

int ox_ee_delta(ox_state *st, double ec_old, double ec_new, double pw1, double pw2,
                double bee, double *out) {
  double EFN = 0., EFO = 0., EEN = 0., EEO = 0.;
  const double ALEEO = pow(ec_old, pw1), ALEEN = pow(ec_new, pw1);
  if (st->p.alphad > 0.0) {
    if (!st->furir_init) {
      snprintf(st->msg, sizeof st->msg, "no k-set yet");
      return MDX_ERR_STATE;
    }
    /* 4.1 reciprocal sum, old and new charges */
    const double ALP2 = st->p.alphad * st->p.alphad;
    const double CFUR = 4.0 * PI * st->p.coulf / st->vol;
    for (int IKV = 1; IKV <= st->nkv; ++IKV) {
      double RXV = st->rkx[IKV] / st->boxl;
      double RYV = st->rky[IKV] / st->boyl;
      double RZV = st->rkz[IKV] / st->bozl;
      double RK2 = RXV * RXV + RYV * RYV + RZV * RZV;
      double SCSO = 0., SSNO = 0., SCSN = 0., SSNN = 0.;
      for (int I = 1; I <= st->nstot; ++I) {
        int IC = st->nsite[I], ITYP = st->itype[I];
        double SCP = RXV * st->sx[I] + RYV * st->sy[I] + RZV * st->sz[I];
        double SSC = sin(SCP), CSC = cos(SCP);
        double QO = st->q[I];
        double QN = st->iee[ITYP] == 0 ? st->charge[IC] * ALEEN : st->q[I];
        SSNO = SSNO + QO * SSC;
        SCSO = SCSO + QO * CSC;
        SSNN = SSNN + QN * SSC;
        SCSN = SCSN + QN * CSC;
      }
      double AKC = CFUR * exp(-0.25 * RK2 / ALP2) / RK2;
      EFO = EFO + (SSNO * SSNO + SCSO * SCSO) * AKC;
      EFN = EFN + (SSNN * SSNN + SCSN * SCSN) * AKC;
    }
    /* 4.2.1 self terms */
    double ABC = st->p.alphad / sqrt(PI);
    for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP)
      if (st->iee[ITYP] == 0)
        for (int II = 1; II <= st->nsits[ITYP]; ++II) {
          int IS = st->isadr[ITYP] + II;
          EFO = EFO - st->p.coulf * (ALEEO * st->charge[IS]) * (ALEEO * st->charge[IS]) * ABC *
                          st->nspec[ITYP];
          EFN = EFN - st->p.coulf * (ALEEN * st->charge[IS]) * (ALEEN * st->charge[IS]) * ABC *
                          st->nspec[ITYP];
        }
    /* 4.2.2 intramolecular terms of EE molecules */
    for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP) {
      if (!(st->iee[ITYP] == 0 && st->nsits[ITYP] > 1)) continue;
      int ISBEG = st->isadr[ITYP] + 1, ISEND = st->isadr[ITYP + 1];
      for (int IS = ISBEG; IS <= ISEND - 1; ++IS)
        for (int JS = IS + 1; JS <= ISEND; ++JS)
          for (int IM = 1; IM <= st->nspec[ITYP]; ++IM) {
            int ISP = st->isaddr[ITYP] + (IM - 1) * st->nsits[ITYP] + IS - ISBEG + 1;
            int JSP = st->isaddr[ITYP] + (IM - 1) * st->nsits[ITYP] + JS - ISBEG + 1;
            double QIJO = st->p.coulf * st->q[ISP] * st->q[JSP];
            double QIJN = st->p.coulf * ALEEN * ALEEN * st->charge[IS] * st->charge[JS];
            double DX = st->sx[ISP] - st->sx[JSP];
            double DY = st->sy[ISP] - st->sy[JSP];
            double DZ = st->sz[ISP] - st->sz[JSP];
            pbc(st, &DX, &DY, &DZ);
            double R2 = DX * DX + DY * DY + DZ * DZ;
            double R2I = 1.0 / R2, R1 = sqrt(R2), R1I = R1 * R2I;
            double ALPHAR = st->p.alphad * R1;
            double TTT = 1.0 / (1.0 + B1 * ALPHAR);
            double EXP2A = exp(-(ALPHAR * ALPHAR));
            double ERFC = ((((A5 * TTT + A4) * TTT + A3) * TTT + A2) * TTT + A1) * TTT * EXP2A;
            double ERFR = (ERFC - 1.0) * R1I;
            EFO = EFO + QIJO * ERFR;
            EFN = EFN + QIJN * ERFR;
          }
    }
  }
  /* DIFEN over the long and the short lists */
  double RSHO = bee * (1. - pow(ec_old, pw2)), RSHN = bee * (1. - pow(ec_new, pw2));
  for (int pass = 0; pass < 2; ++pass) {
    int np = pass == 0 ? st->mbln : st->mbsh;
    const int *L1 = pass == 0 ? st->nbl1 : st->nbs1, *L2 = pass == 0 ? st->nbl2 : st->nbs2;
    for (int INP = 1; INP <= np; ++INP) {
      int ISP = abs(L1[INP]), JSP = L2[INP];
      if (st->iee[st->itype[ISP]] * st->iee[st->itype[JSP]] == 1) continue;
      if (st->nnum[ISP] == st->nnum[JSP]) continue;
      EEO += ee_pair_energy(st, ISP, JSP, ALEEN, RSHO, RSHN, &EEN);
    }
  }
  out[0] = EFN;
  out[1] = EFO;
  out[2] = EEN;
  out[3] = EEO;
  return MDX_OK;
}

/* ---------------------------------------------------------------- RECINT */
int ox_set_lambda(ox_state *st, double ec, double pw1, double pw2,
                  double bee) {
  int nb = st->nnbt;
  st->spei = 0.;
  for (int ITYP = 1; ITYP <= st->ntypes; ++ITYP) {
    double ESCI = st->iee[ITYP] == 0 ? pow(ec, pw1) : 1.0;
    for (int I = st->isadr[ITYP] + 1; I <= st->isadr[ITYP + 1]; ++I) {
      int IS = st->inbt[I];
      for (int JTYP = 1; JTYP <= st->ntypes; ++JTYP) {
        double ESCL = ESCI;
        if (st->iee[JTYP] == 0) ESCL = pow(ec, pw1);
        for (int J = st->isadr[JTYP] + 1; J <= st->isadr[JTYP + 1]; ++J) {
          int JS = st->inbt[J];
          st->a6lj[IDX2(IS, JS, nb)] = ESCL * st->a6lj0[IDX2(IS, JS, nb)];
          st->b12lj[IDX2(IS, JS, nb)] = ESCL * st->b12lj0[IDX2(IS, JS, nb)];
        }
      }
    }
    for (int ISP = st->isaddr[ITYP] + 1; ISP <= st->isaddr[ITYP + 1]; ++ISP)
      st->q[ISP] = ESCI * st->charge[st->nsite[ISP]];
    double SPET = 0.;
    for (int I = 1; I <= st->nsits[ITYP]; ++I) {
      int IS = st->isadr[ITYP] + I;
      double eq = ESCI * st->charge[IS];
      double QII = st->p.coulf * (eq * eq);
      SPET = SPET - st->nspec[ITYP] * st->p.alphad * QII / sqrt(PI);
    }
    st->speei[ITYP] = SPET;
    st->spei = st->spei + SPET;
  }
  st->p.raex = bee * (1. - pow(ec, pw2));
  st->p.ec_me = ec;
  return MDX_OK;
}

/* ------------------------------------------------------------------ PIMD */
/* PIFORCES (pimd.f:321-395) for every bead: harmonic springs to the beads
 * below (JBEAD-1, received first, PI_SENDCOORD(1)) and above (JBEAD+1),
 * whose coordinates arrive as REAL*4 (pimd.f:450-486).  Adds to HX/HY/HZ,
 * VIRFX/Y/Z; returns QEK = 0.5 * sum over beads (the MPI_ALLREDUCE,
 * pimd.f:383-385) and each bead's VIRPI. */
static double piforces(ox_state *const *b, int P, const mdx_pimd_params *pp,
                       double *virpi) {
  double qsum = 0.;
  for (int jb = 0; jb < P; ++jb) {
    ox_state *st = b[jb];
    double QEK = 0.;
    for (int dir = 0; dir < 2; ++dir) {
      const ox_state *o = b[dir == 0 ? (jb + P - 1) % P : (jb + 1) % P];
      double VIRPI = 0.;
      for (int I = 1; I <= st->nstot; ++I) {
        int IS = st->nsite[I];
        double BX = st->sx[I] - (double)(float)o->sx[I];
        double BY = st->sy[I] - (double)(float)o->sy[I];
        double BZ = st->sz[I] - (double)(float)o->sz[I];
        pbc(st, &BX, &BY, &BZ);
        double BSQ = BX * BX + BY * BY + BZ * BZ;
        double BBB = sqrt(BSQ);
        double R1I = 1.0 / BBB;
        double DBND = BBB * pp->beadfac * st->mass[IS];
        double EBDD = DBND * BBB;
        double FORB = -2.0 * DBND * R1I;
        st->hx[I] = st->hx[I] + BX * FORB;
        st->hy[I] = st->hy[I] + BY * FORB;
        st->hz[I] = st->hz[I] + BZ * FORB;
        QEK = QEK + EBDD;
        if (dir == 0) {
          VIRPI = VIRPI + FORB * BSQ;
          st->s.virfx = st->s.virfx + FORB * (BX * BX) * P;
          st->s.virfy = st->s.virfy + FORB * (BY * BY) * P;
          st->s.virfz = st->s.virfz + FORB * (BZ * BZ) * P;
        }
      }
      if (dir == 0) virpi[jb] = VIRPI;
    }
    qsum = qsum + QEK;
  }
  return 0.5 * qsum;
}

/* BEADNOSE (pimd.f:402-444): per atom, the kinetic energy summed over
 * beads drives a Nose-Hoover chain of length JNH shared by the atom's beads;
 * every bead's momentum of that atom is scaled by SCV. */
static void beadnose(ox_state *const *b, int P, const mdx_pimd_params *pp,
                     double *thermo) {
  const ox_state *s0 = b[0];
  const int n = s0->nstot, JNH = pp->jnh;
  const double TSTEB = s0->p.tsteb, TRTEMP = s0->p.trtemp;
  for (int I = 1; I <= n; ++I) {
    double FEK = 0.;
    for (int jb = 0; jb < P; ++jb) {
      const ox_state *st = b[jb];
      FEK = FEK + 0.5 * (st->vx[I] * st->vx[I] + st->vy[I] * st->vy[I] +
                         st->vz[I] * st->vz[I]) * st->massdi[I];
    }
    double *T = thermo + (I - 1); /* THERMO(I, J) at T[(J-1) * n] */
    double ATEMP = FEK * pp->conveq;
    double DKE = ATEMP / TRTEMP - 1.0;
    T[0] = T[0] + DKE * pp->dqqt * TSTEB;
    for (int J = 2; J <= JNH; ++J) {
      T[(size_t)(J - 1) * n] = T[(size_t)(J - 1) * n] +
                               (T[(size_t)(J - 2) * n] * T[(size_t)(J - 2) * n] - pp->fnh) * TSTEB;
      T[(size_t)(J - 2) * n] = T[(size_t)(J - 2) * n] * (1. - T[(size_t)(J - 1) * n] * TSTEB);
    }
    double SCV = 1. - T[0] * TSTEB;
    for (int jb = 0; jb < P; ++jb) {
      ox_state *st = b[jb];
      st->vx[I] = st->vx[I] * SCV;
      st->vy[I] = st->vy[I] * SCV;
      st->vz[I] = st->vz[I] * SCV;
    }
  }
}

static void scale_forces(ox_state *st, int P, int slow) {
  for (int I = 1; I <= st->nstot; ++I) {
    if (slow) {
      st->gx[I] = st->gx[I] / P;
      st->gy[I] = st->gy[I] / P;
      st->gz[I] = st->gz[I] / P;
    }
    st->hx[I] = st->hx[I] / P;
    st->hy[I] = st->hy[I] / P;
    st->hz[I] = st->hz[I] / P;
  }
}

int ox_pimd_steps(ox_state *const *b, const mdx_pimd_params *pp, double *thermo,
                  int32_t nsteps, int32_t mstep0, int prologue, mdx_pimd_record *rec) {
  int rc;
  const int P = pp->nbeads;
  if (P < 2 || pp->jnh < 1) return MDX_ERR_ARG;
  ox_state *s0 = b[0];
  if (s0->p.lnvt || s0->p.lnpt) {
    snprintf(s0->msg, sizeof s0->msg, "PIMD with NVT/NPT scaling is not built");
    return MDX_ERR_UNSUPPORTED;
  }
  double *virpi = (double *)xcalloc((size_t)P, sizeof(double));
  const int NFREQ = s0->p.nfreq, NFREQ2 = NFREQ / 2 + 1;
  const double HTSTEP = 0.5 * s0->p.tstep, TSTEB = s0->p.tsteb, HTSTEB = 0.5 * s0->p.tsteb;
  if (prologue) { /* 1.2 (pimd.f:48-72) */
    for (int jb = 0; jb < P; ++jb) {
      ox_state *st = b[jb];
      st->th.vira[0] = st->th.vira[1] = st->th.vira[2] = 0.;
      if ((rc = ox_chcnb(st, NULL, NULL))) goto out;
      ox_getcom(st);
      if ((rc = ox_slforces(st, NULL))) goto out;
      ox_fforces(st, 0, NULL);
      scale_forces(st, P, 1);
    }
    piforces(b, P, pp, virpi);
  }
  for (int NSTEP = 1; NSTEP <= nsteps; ++NSTEP) {
    const int MSTEP = mstep0 + NSTEP;
    double QEKS = 0.;
    for (int jb = 0; jb < P; ++jb) { /* PI_SCALING(1): GETEMP only (no NVT/NPT) */
      if ((rc = getemp(b[jb]))) goto out;
      kick(b[jb], b[jb]->gx, b[jb]->gy, b[jb]->gz, HTSTEP);
    }
    for (int NSTEB = 1; NSTEB <= NFREQ; ++NSTEB) {
      for (int jb = 0; jb < P; ++jb) kick(b[jb], b[jb]->hx, b[jb]->hy, b[jb]->hz, HTSTEB);
      beadnose(b, P, pp, thermo);
      for (int jb = 0; jb < P; ++jb) {
        ox_state *st = b[jb];
        for (int I = 1; I <= st->nstot; ++I)
          if (st->lmove[st->itype[I]]) {
            st->sx[I] = st->vx[I] * TSTEB * st->massdi[I] + st->sx[I];
            st->sy[I] = st->vy[I] * TSTEB * st->massdi[I] + st->sy[I];
            st->sz[I] = st->vz[I] * TSTEB * st->massdi[I] + st->sz[I];
          }
        ox_getcom(st);
        if (NSTEB == NFREQ2 && MSTEP % st->p.ichnb == 0)
          if ((rc = ox_chcnb(st, NULL, NULL))) goto out;
        if (NSTEB == NFREQ) {
          if ((rc = ox_slforces(st, NULL))) goto out;
          ox_fforces(st, 1, NULL);
          scale_forces(st, P, 1);
        } else {
          ox_fforces(st, 0, NULL);
          scale_forces(st, P, 0);
        }
      }
      QEKS = QEKS + piforces(b, P, pp, virpi);
      for (int jb = 0; jb < P; ++jb) {
        kick(b[jb], b[jb]->hx, b[jb]->hy, b[jb]->hz, HTSTEB);
        if ((rc = getemp(b[jb]))) goto out;
      }
    }
    for (int jb = 0; jb < P; ++jb) {
      kick(b[jb], b[jb]->gx, b[jb]->gy, b[jb]->gz, HTSTEP);
      if ((rc = getemp(b[jb]))) goto out; /* PI_SCALING(2) */
    }
    if (rec) {
      mdx_pimd_record *r = &rec[NSTEP - 1];
      memset(r, 0, sizeof *r);
      r->mstep = MSTEP;
      r->qek = QEKS / NFREQ;
      for (int jb = 0; jb < P; ++jb) {
        const mdx_scalars *s = &b[jb]->s;
        r->virpi += virpi[jb];
        r->pe += s->pe1 + s->pe2 + s->pels1 + s->pels2 + s->spe + s->pint;
        r->tke += b[jb]->th.tke;
        r->temp += b[jb]->th.temp;
      }
      r->temp /= P;
    }
  }
  rc = MDX_OK;
out:
  free(virpi);
  return rc;
}
