/*
 * opaw_oracle.c — CPU FP64 restatement of the OPAW-TDDFT propagation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU library is
 * compared against; it is never linked into, loaded by, or called from the
 * product library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.
 *
 * Every routine restates one subroutine of minhchemucla/OPAW-TDDFT (Fortran
 * 90) and cites the lines it follows.  The reference cannot be compiled on
 * this machine (no Fortran compiler, MPI, FFTW3 or libxc), so parity is
 * pinned by the reference's own known-answer check (the analytic-DFT test of
 * rconv, src/lib/library_rconv_drv.f90:5-95, reproduced in tests/golden) and by
 * the identities its debug routines print (src/test_T.f90, src/test_V.f90,
 * src/nhat.f90:31-41, src/rk4.f90:81-102).  The rest is "parity unpinned".
 *
 * Third-party arithmetic restated from published algorithms:
 *   - FFTW3 (unpinned version): the unnormalised DFT, forward sign -1
 *     (FFTW_FORWARD), backward +1; computed here by a recursive mixed-radix
 *     Cooley-Tukey decomposition.
 *   - libxc LDA_X (id 1) + LDA_C_PW (id 12) (unpinned version): Slater
 *     exchange and the Perdew-Wang 1992 correlation, PRB 45, 13244 (1992),
 *     eqs. (10) and Table I, unpolarised column.
 *
 * Arrays are x fastest (Fortran column-major), 0-based here.  OpenMP
 * parallelises over independent orbitals or grid lines; every reduction runs
 * in a fixed order, so results do not depend on the thread count.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/opaw_gb300.h"

typedef double complex cplx;

/* ------------------------------------------------------------------------ */
/* FFT: recursive mixed-radix Cooley-Tukey, unnormalised                      */
/* ------------------------------------------------------------------------ */

typedef struct {
  int n;
  int nf;
  int f[32];
  cplx *w; /* w[t] = exp(sign * 2 pi i t / n), t in [0, n) */
  int sign;
} fft_plan1;

static void plan1_init(fft_plan1 *p, int n, int sign) {
  p->n = n;
  p->sign = sign;
  p->nf = 0;
  int m = n;
  static const int pref[] = {4, 2, 3, 5, 7};
  for (int k = 0; k < 5 && m > 1; k++) {
    while (m % pref[k] == 0) {
      p->f[p->nf++] = pref[k];
      m /= pref[k];
    }
  }
  for (int q = 11; m > 1; q += 2) {
    while (m % q == 0) {
      p->f[p->nf++] = q;
      m /= q;
    }
  }
  p->w = (cplx *)malloc(sizeof(cplx) * (size_t)(n > 0 ? n : 1));
  for (int t = 0; t < n; t++) {
    double a = 2.0 * M_PI * (double)t / (double)n;
    p->w[t] = cos(a) + (double)sign * sin(a) * I;
  }
}

static void plan1_free(fft_plan1 *p) { free(p->w); }

/* out[k] = sum_j in[j*stride] W^{jk}; scratch holds n elements */
static void fft_rec(const fft_plan1 *p, const cplx *in, int stride, cplx *out, int n, int level,
                    cplx *scratch) {
  if (n == 1) {
    out[0] = in[0];
    return;
  }
  int r = p->f[level];
  int m = n / r;
  /* sub-transforms of the r decimated sequences into out[q*m .. q*m+m) */
  for (int q = 0; q < r; q++) fft_rec(p, in + (size_t)q * stride, stride * r, out + (size_t)q * m, m, level + 1, scratch);
  int step = p->n / n; /* W_n^{t} = W_N^{t*step} */
  cplx t[64];
  cplx *tmp = scratch;
  for (int k = 0; k < m; k++) {
    for (int q = 0; q < r; q++) t[q] = out[(size_t)q * m + k] * p->w[((size_t)q * k * step) % p->n];
    for (int s = 0; s < r; s++) {
      cplx acc = 0;
      for (int q = 0; q < r; q++) acc += t[q] * p->w[((size_t)q * s * m * step) % p->n];
      tmp[k + (size_t)m * s] = acc;
    }
  }
  memcpy(out, tmp, sizeof(cplx) * (size_t)n);
}

/* in-place 3D DFT of a (x fastest) array; sign -1 forward, +1 backward */
void orc_fft3d(int nx, int ny, int nz, cplx *a, int sign) {
  int dims[3] = {nx, ny, nz};
  size_t strides[3] = {1, (size_t)nx, (size_t)nx * ny};
  for (int ax = 0; ax < 3; ax++) {
    int n = dims[ax];
    if (n == 1) continue;
    fft_plan1 p;
    plan1_init(&p, n, sign);
    size_t nlines = (size_t)nx * ny * nz / n;
#pragma omp parallel
    {
      cplx *line = (cplx *)malloc(sizeof(cplx) * n);
      cplx *outl = (cplx *)malloc(sizeof(cplx) * n);
      cplx *scr = (cplx *)malloc(sizeof(cplx) * n);
#pragma omp for schedule(static)
      for (size_t l = 0; l < nlines; l++) {
        /* line l: enumerate the other two indices */
        size_t base;
        if (ax == 0) {
          base = l * (size_t)nx;
        } else if (ax == 1) {
          size_t ix = l % nx, iz = l / nx;
          base = ix + (size_t)nx * ny * iz;
        } else {
          base = l; /* l in [0, nx*ny) */
        }
        for (int j = 0; j < n; j++) line[j] = a[base + strides[ax] * j];
        fft_rec(&p, line, 1, outl, n, 0, scr);
        for (int j = 0; j < n; j++) a[base + strides[ax] * j] = outl[j];
      }
      free(line);
      free(outl);
      free(scr);
    }
    plan1_free(&p);
  }
}

/* ------------------------------------------------------------------------ */
/* context                                                                    */
/* ------------------------------------------------------------------------ */

typedef struct orc_ctx {
  opaw_system sys; /* pointers refer to the copies below */
  int nx, ny, nz;
  size_t nn;
  double dv;
  int natom;
  int *ir_start, *nrough, *ms, *ngrid, *local_grid, *nlm;
  size_t *poff;   /* per atom offset into p3d (ms*nbox) */
  size_t *soff;   /* per atom offset into s/sinv (ms) */
  size_t *doff;   /* per atom offset into ms*ms arrays */
  size_t *goff;   /* per atom offset into local_grid points */
  size_t *g3off;  /* per atom offset into g3d */
  size_t *qoff;   /* per atom offset into qijlm */
  size_t *eoff;   /* per atom offset into eijkl */
  double *p3d, *p3d1, *s, *sinv, *g3d, *qijlm, *vloc, *ncoret, *dij0, *eijkl;
  size_t np, ns, nd, ng;
  double *ek;     /* [nn] kinetic table with 1/nn folded in */
  int nxb, nyb, nzb;
  double *vk;     /* [nb] MT kernel with 1/Nb folded in */
  /* per-set state */
  double *vks[2], *dij[2], *rhoij[2], *dens[2], *nhat[2], *vh[2], *vxc[2];
  /* on-site XC tables (oxc = 0: the term is off) */
  int oxc;
  int *rad_n, *nphi, *proj_lmn;
  size_t *roff, *phioff;
  double *rad_r, *rad_w, *phi, *tphi, *core, *tcore;
} orc_ctx;

static void *dupa(const void *src, size_t bytes) {
  void *p = malloc(bytes ? bytes : 1);
  if (src && bytes) memcpy(p, src, bytes);
  else memset(p, 0, bytes ? bytes : 1);
  return p;
}

void orc_ek_prep(orc_ctx *c);
void orc_vk_prep(orc_ctx *c);

orc_ctx *orc_create(const opaw_system *sys) {
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  c->sys = *sys;
  c->nx = sys->nx;
  c->ny = sys->ny;
  c->nz = sys->nz;
  c->nn = (size_t)c->nx * c->ny * c->nz;
  c->dv = sys->dx * sys->dy * sys->dz;
  int na = c->natom = sys->natom;
  c->ir_start = (int *)dupa(sys->ir_start, sizeof(int) * 3 * na);
  c->nrough = (int *)dupa(sys->nrough, sizeof(int) * 3 * na);
  c->ms = (int *)dupa(sys->ms, sizeof(int) * na);
  c->ngrid = (int *)dupa(sys->ngrid, sizeof(int) * na);
  c->nlm = (int *)dupa(sys->nlm, sizeof(int) * na);
  c->poff = (size_t *)calloc(na + 1, sizeof(size_t));
  c->soff = (size_t *)calloc(na + 1, sizeof(size_t));
  c->doff = (size_t *)calloc(na + 1, sizeof(size_t));
  c->goff = (size_t *)calloc(na + 1, sizeof(size_t));
  c->g3off = (size_t *)calloc(na + 1, sizeof(size_t));
  c->qoff = (size_t *)calloc(na + 1, sizeof(size_t));
  c->eoff = (size_t *)calloc(na + 1, sizeof(size_t));
  for (int a = 0; a < na; a++) {
    size_t nbox = (size_t)c->nrough[3 * a] * c->nrough[3 * a + 1] * c->nrough[3 * a + 2];
    size_t m = c->ms[a];
    c->poff[a + 1] = c->poff[a] + m * nbox;
    c->soff[a + 1] = c->soff[a] + m;
    c->doff[a + 1] = c->doff[a] + m * m;
    c->goff[a + 1] = c->goff[a] + c->ngrid[a];
    c->g3off[a + 1] = c->g3off[a] + (size_t)c->ngrid[a] * c->nlm[a];
    c->qoff[a + 1] = c->qoff[a] + (size_t)c->nlm[a] * m * m;
    c->eoff[a + 1] = c->eoff[a] + m * m * m * m;
  }
  c->np = c->poff[na];
  c->ns = c->soff[na];
  c->nd = c->doff[na];
  c->ng = c->goff[na];
  c->local_grid = (int *)dupa(sys->local_grid, sizeof(int) * 3 * c->ng);
  c->p3d = (double *)dupa(sys->p3d, sizeof(double) * c->np);
  c->p3d1 = (double *)dupa(sys->p3d1, sizeof(double) * c->np);
  c->s = (double *)dupa(sys->s, sizeof(double) * c->ns);
  c->sinv = (double *)dupa(sys->sinv, sizeof(double) * c->ns);
  c->g3d = (double *)dupa(sys->g3d, sizeof(double) * c->g3off[na]);
  c->qijlm = (double *)dupa(sys->qijlm, sizeof(double) * c->qoff[na]);
  c->vloc = (double *)dupa(sys->vloc, sizeof(double) * c->nn);
  c->ncoret = (double *)dupa(sys->ncoret, sizeof(double) * c->nn);
  c->dij0 = (double *)dupa(sys->dij0, sizeof(double) * c->nd);
  c->eijkl = (double *)dupa(sys->eijkl, sizeof(double) * c->eoff[na]);
  for (int s = 0; s < 2; s++) {
    c->vks[s] = (double *)calloc(c->nn, sizeof(double));
    c->dens[s] = (double *)calloc(c->nn, sizeof(double));
    c->nhat[s] = (double *)calloc(c->nn, sizeof(double));
    c->vh[s] = (double *)calloc(c->nn, sizeof(double));
    c->vxc[s] = (double *)calloc(c->nn, sizeof(double));
    c->dij[s] = (double *)calloc(c->nd ? c->nd : 1, sizeof(double));
    c->rhoij[s] = (double *)calloc(c->nd ? c->nd : 1, sizeof(double));
  }
  if (sys->rad_n) {
    c->oxc = 1;
    c->rad_n = (int *)dupa(sys->rad_n, sizeof(int) * na);
    c->nphi = (int *)dupa(sys->nphi, sizeof(int) * na);
    c->proj_lmn = (int *)dupa(sys->proj_lmn, sizeof(int) * 3 * c->ns);
    c->roff = (size_t *)calloc(na + 1, sizeof(size_t));
    c->phioff = (size_t *)calloc(na + 1, sizeof(size_t));
    for (int a = 0; a < na; a++) {
      c->roff[a + 1] = c->roff[a] + c->rad_n[a];
      c->phioff[a + 1] = c->phioff[a] + (size_t)c->nphi[a] * c->rad_n[a];
    }
    c->rad_r = (double *)dupa(sys->rad_r, sizeof(double) * c->roff[na]);
    c->rad_w = (double *)dupa(sys->rad_w, sizeof(double) * c->roff[na]);
    c->core = (double *)dupa(sys->coredens, sizeof(double) * c->roff[na]);
    c->tcore = (double *)dupa(sys->tcoredens, sizeof(double) * c->roff[na]);
    c->phi = (double *)dupa(sys->phi, sizeof(double) * c->phioff[na]);
    c->tphi = (double *)dupa(sys->tphi, sizeof(double) * c->phioff[na]);
  }
  orc_ek_prep(c);
  orc_vk_prep(c);
  return c;
}

void orc_free(orc_ctx *c) {
  if (!c) return;
  void *ps[] = {c->ir_start, c->nrough, c->ms, c->ngrid, c->nlm, c->poff, c->soff, c->doff,
                c->goff, c->g3off, c->qoff, c->eoff, c->local_grid, c->p3d, c->p3d1, c->s,
                c->sinv, c->g3d, c->qijlm, c->vloc, c->ncoret, c->dij0, c->eijkl, c->ek, c->vk};
  for (size_t i = 0; i < sizeof(ps) / sizeof(ps[0]); i++) free(ps[i]);
  void *po[] = {c->rad_n, c->nphi, c->proj_lmn, c->roff, c->phioff, c->rad_r, c->rad_w, c->core, c->tcore,
                c->phi, c->tphi};
  for (size_t i = 0; i < sizeof(po) / sizeof(po[0]); i++) free(po[i]);
  for (int s = 0; s < 2; s++) {
    free(c->vks[s]); free(c->dens[s]); free(c->nhat[s]); free(c->vh[s]);
    free(c->vxc[s]); free(c->dij[s]); free(c->rhoij[s]);
  }
  free(c);
}

/* state accessors */
void orc_set_vks(orc_ctx *c, int set, const double *v) { memcpy(c->vks[set], v, sizeof(double) * c->nn); }
void orc_get_vks(orc_ctx *c, int set, double *v) { memcpy(v, c->vks[set], sizeof(double) * c->nn); }
void orc_set_dij(orc_ctx *c, int set, const double *d) { memcpy(c->dij[set], d, sizeof(double) * c->nd); }
void orc_get_dij(orc_ctx *c, int set, double *d) { memcpy(d, c->dij[set], sizeof(double) * c->nd); }
void orc_get_rhoij(orc_ctx *c, int set, double *d) { memcpy(d, c->rhoij[set], sizeof(double) * c->nd); }
void orc_get_density(orc_ctx *c, int set, double *d) { memcpy(d, c->dens[set], sizeof(double) * c->nn); }
void orc_get_nhat(orc_ctx *c, int set, double *d) { memcpy(d, c->nhat[set], sizeof(double) * c->nn); }
void orc_get_vh(orc_ctx *c, int set, double *d) { memcpy(d, c->vh[set], sizeof(double) * c->nn); }
void orc_get_vxc(orc_ctx *c, int set, double *d) { memcpy(d, c->vxc[set], sizeof(double) * c->nn); }
void orc_get_ek(orc_ctx *c, double *d) { memcpy(d, c->ek, sizeof(double) * c->nn); }
void orc_get_vk(orc_ctx *c, double *d) { memcpy(d, c->vk, sizeof(double) * (size_t)c->nxb * c->nyb * c->nzb); }

/* ------------------------------------------------------------------------ */
/* A15 kinetic table: ek.f90:18-50 (Gamma point, nk_loc = 1)                  */
/* ------------------------------------------------------------------------ */
static double kcomp(int i, int n, double d) {
  double pi = acos(-1.0);
  double dk = 2.0 * pi / (n * d);    /* ek.f90:18 */
  double k = (double)i * dk;         /* ek.f90:26 */
  if (k > pi / d) k = k - 2.0 * pi / d; /* ek.f90:30 */
  return k;
}

void orc_ek_prep(orc_ctx *c) {
  c->ek = (double *)malloc(sizeof(double) * c->nn);
  double ekcut = c->sys.ekcut;
  for (int iz = 0; iz < c->nz; iz++)
    for (int iy = 0; iy < c->ny; iy++)
      for (int ix = 0; ix < c->nx; ix++) {
        double kx = kcomp(ix, c->nx, c->sys.dx), ky = kcomp(iy, c->ny, c->sys.dy),
               kz = kcomp(iz, c->nz, c->sys.dz);
        double e = (kx * kx + ky * ky + kz * kz) / 2.0; /* ek.f90:40 */
        if (ekcut > 0 && e > ekcut) e = ekcut;          /* ek.f90:42-44 */
        c->ek[ix + (size_t)c->nx * (iy + (size_t)c->ny * iz)] =
            e / ((double)c->nx * (double)c->ny * (double)c->nz); /* ek.f90:50 */
      }
}

/* ------------------------------------------------------------------------ */
/* A14 Martyna-Tuckerman kernel: vk_scale.f90:23-48 + vk_TuMa.f90:2-117       */
/* ------------------------------------------------------------------------ */
void orc_vk_prep(orc_ctx *c) {
  int sv = c->sys.scale_vh > 0 ? c->sys.scale_vh : 1;
  int nx = c->nxb = sv * c->nx, ny = c->nyb = sv * c->ny, nz = c->nzb = sv * c->nz;
  double dx = c->sys.dx, dy = c->sys.dy, dz = c->sys.dz;
  size_t nb = (size_t)nx * ny * nz;
  double pi = acos(-1.0);
  cplx *cvk = (cplx *)calloc(nb, sizeof(cplx));
  double lx = nx * dx, ly = ny * dy, lz = nz * dz;
  double lmin = lx < ly ? lx : ly;
  if (lz < lmin) lmin = lz;
  double aa = 7.0 / lmin;                                      /* vk_TuMa.f90:25 */
  double r0[3] = {-(nx) / 2.0 * dx, -(ny) / 2.0 * dy, -(nz) / 2.0 * dz}; /* :26 */
  double dvb = dx * dy * dz;
  double dkx = 2.0 * pi / ((double)nx * dx), dky = 2.0 * pi / ((double)ny * dy),
         dkz = 2.0 * pi / ((double)nz * dz);
  if (!c->sys.periodic) {
    for (int iz = 0; iz < nz; iz++)
      for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++) {
          double rx = r0[0] + ix * dx, ry = r0[1] + iy * dy, rz = r0[2] + iz * dz;
          double r2 = rx * rx + ry * ry + rz * rz;
          double floor2 = (double)1e-26f; /* single-precision literal at :51 */
          double rp = sqrt(r2 > floor2 ? r2 : floor2);
          cvk[ix + (size_t)nx * (iy + (size_t)ny * iz)] = erf(aa * rp) / rp * dvb; /* :52 */
        }
    /* fft3d_general(.,1) = conj(fft_forward(conj(.))): unnormalised backward */
    orc_fft3d(nx, ny, nz, cvk, +1);
  }
  for (int iz = 0; iz < nz; iz++)
    for (int iy = 0; iy < ny; iy++)
      for (int ix = 0; ix < nx; ix++) {
        double kx = ix * dkx, ky = iy * dky, kz = iz * dkz; /* :65-67 */
        if (kx > pi / dx) kx = kx - 2.0 * pi / dx;
        if (ky > pi / dy) ky = ky - 2.0 * pi / dy;
        if (kz > pi / dz) kz = kz - 2.0 * pi / dz;
        double k2 = kx * kx + ky * ky + kz * kz;
        size_t i = ix + (size_t)nx * (iy + (size_t)ny * iz);
        cplx cterm;
        if (!c->sys.periodic) {
          double ph = r0[0] * kx + r0[1] * ky + r0[2] * kz;
          cvk[i] = cvk[i] * (cos(ph) + sin(ph) * I); /* :77-78 */
          double k2s = k2 / (4.0 * aa * aa);
          if (k2s > 1e-8)
            cterm = 4.0 * pi / k2 * (1.0 - exp(-k2s)); /* :85 */
          else
            cterm = 4.0 * pi / (4.0 * aa * aa) * (1.0 - 0.5 * k2s + k2s * k2s / 6.0); /* :88 */
        } else {
          cterm = (k2 > 1e-8) ? 4.0 * pi / k2 : 0.0; /* :93-97 */
        }
        cvk[i] += cterm;
      }
  c->vk = (double *)malloc(sizeof(double) * nb);
  for (size_t i = 0; i < nb; i++) c->vk[i] = creal(cvk[i]) / (double)nx / (double)ny / (double)nz; /* vk_scale.f90:46 */
  free(cvk);
}

/* ------------------------------------------------------------------------ */
/* A2/A3 proj, proj1: proj.f90:19-43, proj1.f90:19-45                         */
/* ------------------------------------------------------------------------ */
static inline size_t gidx(const orc_ctx *c, int a, int bx, int by, int bz) {
  /* 1-based ir_start; periodic wrap of the edge branch (proj.f90:30-32) is
   * the identity for boxes inside the grid */
  int ix = c->ir_start[3 * a] - 1 + bx, iy = c->ir_start[3 * a + 1] - 1 + by,
      iz = c->ir_start[3 * a + 2] - 1 + bz;
  ix = ((ix % c->nx) + c->nx) % c->nx;
  iy = ((iy % c->ny) + c->ny) % c->ny;
  iz = ((iz % c->nz) + c->nz) % c->nz;
  return ix + (size_t)c->nx * (iy + (size_t)c->ny * iz);
}

/* ca[i] = dv * sum_box conj(p_i) * pin ; which 0 = p~ (proj), 1 = p1 (proj1) */
void orc_proj(const orc_ctx *c, int a, int which, const cplx *pin, cplx *ca) {
  const double *P = (which ? c->p3d1 : c->p3d) + c->poff[a];
  int n0 = c->nrough[3 * a], n1 = c->nrough[3 * a + 1], n2 = c->nrough[3 * a + 2];
  size_t nbox = (size_t)n0 * n1 * n2;
  for (int i = 0; i < c->ms[a]; i++) {
    cplx acc = 0;
    size_t b = 0;
    for (int bz = 0; bz < n2; bz++)
      for (int by = 0; by < n1; by++)
        for (int bx = 0; bx < n0; bx++, b++) acc += pin[gidx(c, a, bx, by, bz)] * P[i * nbox + b];
    ca[i] = acc * c->dv;
  }
}

/* scatter: sp[box] += sum_i P_i * coef_i */
static void box_add(const orc_ctx *c, int a, const double *P, const cplx *coef, cplx *sp) {
  int n0 = c->nrough[3 * a], n1 = c->nrough[3 * a + 1], n2 = c->nrough[3 * a + 2];
  size_t nbox = (size_t)n0 * n1 * n2;
  size_t b = 0;
  for (int bz = 0; bz < n2; bz++)
    for (int by = 0; by < n1; by++)
      for (int bx = 0; bx < n0; bx++, b++) {
        cplx acc = 0;
        for (int i = 0; i < c->ms[a]; i++) acc += P[i * nbox + b] * coef[i];
        sp[gidx(c, a, bx, by, bz)] += acc;
      }
}

/* ------------------------------------------------------------------------ */
/* A4 sn_phi: snphi.f90:14-48                                                 */
/* ------------------------------------------------------------------------ */
void orc_sn_phi(const orc_ctx *c, double n, const cplx *pin, cplx *sp) {
  memcpy(sp, pin, sizeof(cplx) * c->nn); /* :14 */
  cplx ca[64], coef[64];
  for (int a = 0; a < c->natom; a++) {
    orc_proj(c, a, 1, pin, ca); /* :23 proj1 of the unmodified input */
    for (int i = 0; i < c->ms[a]; i++) {
      double sn = (n == -1.0) ? c->sinv[c->soff[a] + i] : pow(1.0 + c->s[c->soff[a] + i], n) - 1.0; /* :24-28 */
      coef[i] = sn * ca[i];
    }
    box_add(c, a, c->p3d1 + c->poff[a], coef, sp); /* :29-46 */
  }
}

/* ------------------------------------------------------------------------ */
/* A1 h_phi / h_phi_pert: hphi.f90:14-65                                      */
/* ------------------------------------------------------------------------ */
void orc_h_phi(const orc_ctx *c, int set, const cplx *pin, cplx *hp) {
  size_t nn = c->nn;
  cplx *tmp = (cplx *)malloc(sizeof(cplx) * nn);
  memcpy(tmp, pin, sizeof(cplx) * nn);
  orc_fft3d(c->nx, c->ny, c->nz, tmp, -1);          /* :16 */
  for (size_t i = 0; i < nn; i++) tmp[i] *= c->ek[i]; /* :17 */
  orc_fft3d(c->nx, c->ny, c->nz, tmp, +1);          /* :18 */
  const double *v = c->vks[set];
  for (size_t i = 0; i < nn; i++) hp[i] = tmp[i] + pin[i] * v[i]; /* :21 */
  free(tmp);
  cplx ca[64], arr[64];
  for (int a = 0; a < c->natom; a++) { /* addvnl :31-64 */
    int m = c->ms[a];
    orc_proj(c, a, 0, pin, ca);
    const double *D = c->dij[set] + c->doff[a];
    for (int i = 0; i < m; i++) {
      cplx acc = 0;
      for (int j = 0; j < m; j++) acc += D[i + (size_t)m * j] * ca[j]; /* sum(dij(is,:)*ca(:)) */
      arr[i] = acc;
    }
    box_add(c, a, c->p3d + c->poff[a], arr, hp);
  }
}

/* ------------------------------------------------------------------------ */
/* A5 shs / shs_pert: shs.f90:19-22                                           */
/* ------------------------------------------------------------------------ */
void orc_shs(const orc_ctx *c, int set, const cplx *pin, cplx *pout) {
  cplx *tmp = (cplx *)malloc(sizeof(cplx) * c->nn);
  orc_sn_phi(c, -0.5, pin, tmp);
  orc_h_phi(c, set, tmp, pout);
  memcpy(tmp, pout, sizeof(cplx) * c->nn);
  orc_sn_phi(c, -0.5, tmp, pout);
  free(tmp);
}

/* batched twins (orbitals independent; OpenMP over orbitals) */
void orc_h_phi_batch(const orc_ctx *c, int set, const cplx *pin, cplx *hp, int norb) {
  for (int b = 0; b < norb; b++) orc_h_phi(c, set, pin + (size_t)b * c->nn, hp + (size_t)b * c->nn);
}
void orc_sn_phi_batch(const orc_ctx *c, double n, const cplx *pin, cplx *sp, int norb) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < norb; b++) orc_sn_phi(c, n, pin + (size_t)b * c->nn, sp + (size_t)b * c->nn);
}
void orc_shs_batch(const orc_ctx *c, int set, const cplx *pin, cplx *pout, int norb) {
  for (int b = 0; b < norb; b++) orc_shs(c, set, pin + (size_t)b * c->nn, pout + (size_t)b * c->nn);
}
void orc_proj_batch(const orc_ctx *c, int which, const cplx *pin, int norb, cplx *ca) {
  size_t tot = c->ns;
  for (int b = 0; b < norb; b++)
    for (int a = 0; a < c->natom; a++) orc_proj(c, a, which, pin + (size_t)b * c->nn, ca + b * tot + c->soff[a]);
}

/* ------------------------------------------------------------------------ */
/* A8 tddft_rhoij_2: tddft_rhoij.f90:75-115 (all orbitals occupied, wk = 1)   */
/* ------------------------------------------------------------------------ */
void orc_rhoij(orc_ctx *c, int set, const cplx *psit, int norb) {
  double *R = c->rhoij[set];
  memset(R, 0, sizeof(double) * c->nd);
  cplx ca[64];
  for (int a = 0; a < c->natom; a++) {
    int m = c->ms[a];
    double *Ra = R + c->doff[a];
    for (int b = 0; b < norb; b++) {
      orc_proj(c, a, 0, psit + (size_t)b * c->nn, ca); /* raw p~ (:30) */
      for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++) Ra[i + (size_t)m * j] += creal(conj(ca[i]) * ca[j] * 2.0); /* :35,38 */
    }
  }
}

/* ------------------------------------------------------------------------ */
/* A10 tddft_dens_2: tddft_dens.f90:56-77                                     */
/* ------------------------------------------------------------------------ */
void orc_density(orc_ctx *c, int set, const cplx *psit, int norb) {
  double *d = c->dens[set];
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < c->nn; i++) {
    double acc = 0;
    for (int b = 0; b < norb; b++) {
      cplx z = psit[(size_t)b * c->nn + i];
      acc += creal(z) * creal(z) + cimag(z) * cimag(z);
    }
    d[i] = 2.0 * acc;
  }
}

/* ------------------------------------------------------------------------ */
/* A11 get_nhat / get_nhat_pert: nhat.f90:11-41, nhat_pert.f90                */
/* ------------------------------------------------------------------------ */
void orc_nhat(orc_ctx *c, int set) {
  double *nh = c->nhat[set];
  memset(nh, 0, sizeof(double) * c->nn);
  for (int a = 0; a < c->natom; a++) {
    int m = c->ms[a], L = c->nlm[a], ng = c->ngrid[a];
    const double *R = c->rhoij[set] + c->doff[a];
    const double *Q = c->qijlm + c->qoff[a];
    const double *G = c->g3d + c->g3off[a];
    const int *lg = c->local_grid + 3 * c->goff[a];
    for (int ig = 0; ig < ng; ig++) {
      size_t gi = (lg[3 * ig] - 1) + (size_t)c->nx * ((lg[3 * ig + 1] - 1) + (size_t)c->ny * (lg[3 * ig + 2] - 1));
      for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++)
          for (int l = 0; l < L; l++)
            nh[gi] += R[i + (size_t)m * j] * Q[l + (size_t)L * (i + (size_t)m * j)] * G[ig + (size_t)ng * l]; /* :22-23 */
    }
  }
  /* charge renormalisation (:31-41) */
  double sa = 0, sb = 0;
  for (size_t i = 0; i < c->nn; i++) { sa += nh[i]; sb += c->dens[set][i]; }
  sa *= c->dv;
  sb *= c->dv;
  double f = c->sys.rnel / (sa + sb);
  for (size_t i = 0; i < c->nn; i++) { nh[i] *= f; c->dens[set][i] *= f; }
}

/* ------------------------------------------------------------------------ */
/* A17 LDA: libxc LDA_X + LDA_C_PW (vxc_libxc.f90:15-23, libxc1.f90:46-64)    */
/* ------------------------------------------------------------------------ */
double orc_vxc_point(double n) {
  if (!(n > 1e-15)) return 0.0; /* below the density threshold: no potential */
  double pi = acos(-1.0);
  /* Slater exchange: v_x = -(3 n / pi)^(1/3) */
  double vx = -cbrt(3.0 * n / pi);
  /* PW92 correlation, unpolarised: A, alpha1, beta1..4, p = 1 */
  const double A = 0.031091, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382, b4 = 0.49294;
  double rs = cbrt(3.0 / (4.0 * pi * n));
  double srs = sqrt(rs);
  double Q = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  double dQ = 2.0 * A * (0.5 * b1 / srs + b2 + 1.5 * b3 * srs + 2.0 * b4 * rs);
  double lg = log(1.0 + 1.0 / Q);
  double ec = -2.0 * A * (1.0 + a1 * rs) * lg;
  double dec = -2.0 * A * a1 * lg + 2.0 * A * (1.0 + a1 * rs) * dQ / (Q * Q + Q);
  double vc = ec - rs / 3.0 * dec;
  return vx + vc;
}

void orc_vxc(const double *n, double *v, size_t cnt) {
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < cnt; i++) v[i] = orc_vxc_point(n[i]);
}

/* ------------------------------------------------------------------------ */
/* rconv: library_vh_convolution_r8_r2c.f90:13-31 (r2c == c2c of real data)  */
/* ------------------------------------------------------------------------ */
void orc_rconv(int nx, int ny, int nz, const double *gin, const double *bk, double *gout) {
  size_t n = (size_t)nx * ny * nz;
  cplx *a = (cplx *)malloc(sizeof(cplx) * n);
  for (size_t i = 0; i < n; i++) a[i] = gin[i];
  orc_fft3d(nx, ny, nz, a, -1);
  for (size_t i = 0; i < n; i++) a[i] *= bk[i];
  orc_fft3d(nx, ny, nz, a, +1);
  double cn = 1.0 / ((double)nx * (double)ny * (double)nz);
  for (size_t i = 0; i < n; i++) gout[i] = creal(a[i]) * cn;
  free(a);
}

/* ------------------------------------------------------------------------ */
/* A13 vh_sub: vh_big.f90:11-71 + get_vcon library_fft3d_extra.f90:8-21       */
/* ------------------------------------------------------------------------ */
void orc_vh(const orc_ctx *c, const double *dens, double *vh) {
  int nxb = c->nxb, nyb = c->nyb, nzb = c->nzb;
  size_t nb = (size_t)nxb * nyb * nzb;
  double *db = (double *)calloc(nb, sizeof(double));
  double *vb = (double *)malloc(sizeof(double) * nb);
  int mx = nxb / 2 - c->nx / 2, my = nyb / 2 - c->ny / 2, mz = nzb / 2 - c->nz / 2; /* :44-50, 0-based */
  for (int iz = 0; iz < c->nz; iz++)
    for (int iy = 0; iy < c->ny; iy++)
      for (int ix = 0; ix < c->nx; ix++)
        db[(ix + mx) + (size_t)nxb * ((iy + my) + (size_t)nyb * (iz + mz))] =
            dens[ix + (size_t)c->nx * (iy + (size_t)c->ny * iz)];
  orc_rconv(nxb, nyb, nzb, db, c->vk, vb);
  double nbd = (double)nxb * (double)nyb * (double)nzb;
  for (int iz = 0; iz < c->nz; iz++)
    for (int iy = 0; iy < c->ny; iy++)
      for (int ix = 0; ix < c->nx; ix++)
        vh[ix + (size_t)c->nx * (iy + (size_t)c->ny * iz)] =
            vb[(ix + mx) + (size_t)nxb * ((iy + my) + (size_t)nyb * (iz + mz))] * nbd; /* get_vcon :20 */
  free(db);
  free(vb);
}

/* ------------------------------------------------------------------------ */
/* A12 get_pot_tddft_2: tddft_pot.f90:130-147                                 */
/* ------------------------------------------------------------------------ */
void orc_vks(orc_ctx *c, int set) {
  size_t nn = c->nn;
  double *t = (double *)malloc(sizeof(double) * nn);
  for (size_t i = 0; i < nn; i++) t[i] = c->dens[set][i] + c->ncoret[i];
  orc_vxc(t, c->vxc[set], nn); /* :75-78 */
  for (size_t i = 0; i < nn; i++) t[i] = c->dens[set][i] + c->nhat[set][i];
  orc_vh(c, t, c->vh[set]); /* :39-40 */
  if (c->sys.periodic) {     /* :42-45 */
    double m = 0;
    for (size_t i = 0; i < nn; i++) m += c->vh[set][i];
    m /= (double)nn;
    for (size_t i = 0; i < nn; i++) c->vh[set][i] -= m;
  }
  for (size_t i = 0; i < nn; i++) c->vks[set][i] = c->vh[set][i] + c->vxc[set][i] + c->vloc[i]; /* :46-47 */
  free(t);
}

/* ------------------------------------------------------------------------ */
/* A16 on-site XC term of libpaw's D_ij (pawdenpot + pawdij with pawxcdev = 1, */
/* LDA, nspden = 1, usexcnhat = 0; 2_m_pawxc.F90 pawxcm, 4_m_pawdij.F90       */
/* pawdijxcm): one-centre densities in moments of the real Y_lm               */
/*   n_L(r) = sum_ij rho_ij u_i u_j / r^2 G^L_ij (+ sqrt(4 pi) n_c, L = 0)      */
/* potential moments of the first-order development around n_s = n_0/sqrt4pi */
/*   V_0 = sqrt(4pi) v(n_s) + v''(n_s) sum_{L>0} n_L^2 / (2 sqrt(4pi)),        */
/*   V_L = v'(n_s) n_L,  v', v'' central differences, relative step 1e-4,     */
/* and D_xc_ij = sum_L G^L_ij int (V_L u_i u_j - V~_L u~_i u~_j) dr.           */
/* ------------------------------------------------------------------------ */
static void orc_ylm2(double x, double y, double z, double *Y) {
  /* real spherical harmonics, l <= 2, index l^2 + l + m (ylm.f90 order) */
  const double pi = acos(-1.0);
  Y[0] = sqrt(1.0 / (4.0 * pi));
  Y[1] = sqrt(3.0 / (4.0 * pi)) * y;
  Y[2] = sqrt(3.0 / (4.0 * pi)) * z;
  Y[3] = sqrt(3.0 / (4.0 * pi)) * x;
  Y[4] = sqrt(15.0 / (4.0 * pi)) * x * y;
  Y[5] = sqrt(15.0 / (4.0 * pi)) * y * z;
  Y[6] = sqrt(5.0 / (16.0 * pi)) * (3.0 * z * z - 1.0);
  Y[7] = sqrt(15.0 / (4.0 * pi)) * x * z;
  Y[8] = sqrt(15.0 / (16.0 * pi)) * (x * x - y * y);
}

/* G[L][a][b] = int Y_L Y_a Y_b dOmega, L < 9, a, b < 4: Gauss-Legendre in
 * cos(theta) (16 nodes, Newton on P_16) times 32 uniform points in phi,
 * exact for these polynomial degrees */
static void orc_gaunt(double *G) {
  const int nt = 16, np = 32;
  const double pi = acos(-1.0);
  for (int e = 0; e < 9 * 16; e++) G[e] = 0.0;
  for (int i = 0; i < nt; i++) {
    double t = cos(pi * (i + 0.75) / (nt + 0.5)), d = 1.0, p0 = 1.0, p1 = t;
    for (int it = 0; it < 100; it++) {
      p0 = 1.0;
      p1 = t;
      for (int k = 2; k <= nt; k++) {
        double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      d = nt * (t * p1 - p0) / (t * t - 1.0);
      double dt = p1 / d;
      t -= dt;
      if (fabs(dt) < 1e-16) break;
    }
    double wt = 2.0 / ((1.0 - t * t) * d * d), st = sqrt(1.0 - t * t);
    for (int j = 0; j < np; j++) {
      double ph = 2.0 * pi * j / np, Y[9];
      orc_ylm2(st * cos(ph), st * sin(ph), t, Y);
      for (int L = 0; L < 9; L++)
        for (int a = 0; a < 4; a++)
          for (int b = 0; b < 4; b++) G[(L * 4 + a) * 4 + b] += wt * (2.0 * pi / np) * Y[L] * Y[a] * Y[b];
    }
  }
}

/* v(n0 + dn) - v(n0) by divided differences of every factor of the LDA
 * formula (no cancellation of two nearly equal potentials) */
static void orc_parts(double n, double *u, double *rs, double *s, double *Q, double *dQ, double *lg) {
  const double A = 0.031091, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382, b4 = 0.49294;
  *u = cbrt(n);
  *rs = cbrt(3.0 / (4.0 * acos(-1.0))) / *u;
  *s = sqrt(*rs);
  *Q = 2.0 * A * (b1 * *s + b2 * *rs + b3 * *rs * *s + b4 * *rs * *rs);
  *dQ = 2.0 * A * (0.5 * b1 / *s + b2 + 1.5 * b3 * *s + 2.0 * b4 * *rs);
  *lg = log1p(1.0 / *Q);
}
static double orc_vdiff(double n0, double dn) {
  const double A = 0.031091, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382, b4 = 0.49294;
  double n1 = n0 + dn;
  if (!(n0 > 1e-15) || !(n1 > 1e-15)) return orc_vxc_point(n1) - orc_vxc_point(n0);
  double u0, r0, s0, Q0, dQ0, l0, u1, r1, s1, Q1, dQ1, l1;
  orc_parts(n0, &u0, &r0, &s0, &Q0, &dQ0, &l0);
  orc_parts(n1, &u1, &r1, &s1, &Q1, &dQ1, &l1);
  double du = dn / (u1 * u1 + u1 * u0 + u0 * u0);
  double dvx = -cbrt(3.0 / acos(-1.0)) * du;
  double drs = -cbrt(3.0 / (4.0 * acos(-1.0))) * du / (u1 * u0);
  double ds = drs / (s1 + s0);
  double drss = drs * s1 + r0 * ds, drs2 = drs * (r1 + r0);
  double dQ = 2.0 * A * (b1 * ds + b2 * drs + b3 * drss + b4 * drs2);
  double ddQ = 2.0 * A * (-0.5 * b1 * ds / (s1 * s0) + 1.5 * b3 * ds + 2.0 * b4 * drs);
  double dlg = log1p(-dQ / (Q1 * (Q0 + 1.0)));
  double dec = -2.0 * A * (a1 * drs * l1 + (1.0 + a1 * r0) * dlg);
  double G0 = Q0 * (Q0 + 1.0), G1 = Q1 * (Q1 + 1.0);
  double F1 = dQ1 / G1;
  double dF = (ddQ * G0 - dQ0 * dQ * (Q1 + Q0 + 1.0)) / (G1 * G0);
  double ddec = -2.0 * A * a1 * dlg + 2.0 * A * (a1 * drs * F1 + (1.0 + a1 * r0) * dF);
  double dec1 = -2.0 * A * a1 * l1 + 2.0 * A * (1.0 + a1 * r1) * dQ1 / (Q1 * (Q1 + 1.0));
  return dvx + dec - (drs * dec1 + r0 * ddec) / 3.0;
}

void orc_onsite_xc(orc_ctx *c, const double *rho, double *dxc) {
  double gl[9 * 16];
  orc_gaunt(gl);
  const double sq4pi = sqrt(4.0 * acos(-1.0)), delta = 1e-4;
  for (int a = 0; a < c->natom; a++) {
    int m = c->ms[a], nr = c->rad_n[a];
    const double *R = rho + c->doff[a], *r = c->rad_r + c->roff[a], *w = c->rad_w + c->roff[a];
    const int *lmn = c->proj_lmn + 3 * c->soff[a];
    double *V = (double *)calloc((size_t)2 * 9 * nr, sizeof(double));
    for (int sdx = 0; sdx < 2; sdx++) {
      const double *U = (sdx ? c->tphi : c->phi) + c->phioff[a];
      const double *core = (sdx ? c->tcore : c->core) + c->roff[a];
      for (int k = 0; k < nr; k++) {
        double n[9] = {0};
        for (int i = 0; i < m; i++)
          for (int j = 0; j < m; j++) {
            int ai = lmn[3 * i] * lmn[3 * i] + lmn[3 * i] + lmn[3 * i + 1];
            int aj = lmn[3 * j] * lmn[3 * j] + lmn[3 * j] + lmn[3 * j + 1];
            double f = R[i + (size_t)m * j] * U[(size_t)lmn[3 * i + 2] * nr + k] * U[(size_t)lmn[3 * j + 2] * nr + k] /
                       (r[k] * r[k]);
            for (int L = 0; L < 9; L++) n[L] += f * gl[(L * 4 + ai) * 4 + aj];
          }
        n[0] += sq4pi * core[k];
        double up = 0.5 * n[0] / sq4pi; /* spin density, kept >= xc_denpos */
        if (up < 1e-14) up = 1e-14;
        double ns = 2.0 * up, v0 = orc_vxc_point(ns), h = (ns + delta * ns) - ns, d1 = 0.0, d2 = 0.0; /* ns +- h exact */
        if (up > 1e-14) { /* (v+ - v-) / 2h, (v+ + v- - 2 v0) / h^2 from dp = v+ - v0, dm = v0 - v- */
          double dp = orc_vdiff(ns, h), dm = -orc_vdiff(ns, -h);
          d1 = (dp + dm) / (2.0 * h);
          d2 = (dp - dm) / (h * h);
        }
        double v1 = 0.0;
        for (int L = 1; L < 9; L++) v1 += n[L] * n[L];
        double *Vs = V + (size_t)sdx * 9 * nr;
        Vs[k] = v0 * sq4pi + v1 * d2 / (2.0 * sq4pi);
        for (int L = 1; L < 9; L++) Vs[(size_t)L * nr + k] = d1 * n[L];
      }
    }
    const double *U0 = c->phi + c->phioff[a], *U1 = c->tphi + c->phioff[a];
    for (int j = 0; j < m; j++)
      for (int i = 0; i <= j; i++) {
        int ai = lmn[3 * i] * lmn[3 * i] + lmn[3 * i] + lmn[3 * i + 1];
        int aj = lmn[3 * j] * lmn[3 * j] + lmn[3 * j] + lmn[3 * j + 1];
        double acc = 0.0;
        for (int k = 0; k < nr; k++) {
          double pp = U0[(size_t)lmn[3 * i + 2] * nr + k] * U0[(size_t)lmn[3 * j + 2] * nr + k];
          double tt = U1[(size_t)lmn[3 * i + 2] * nr + k] * U1[(size_t)lmn[3 * j + 2] * nr + k];
          double sm = 0.0;
          for (int L = 0; L < 9; L++)
            sm += gl[(L * 4 + ai) * 4 + aj] * (V[(size_t)L * nr + k] * pp - V[(size_t)(9 + L) * nr + k] * tt);
          acc += w[k] * sm;
        }
        dxc[c->doff[a] + i + (size_t)m * j] = acc;
        dxc[c->doff[a] + j + (size_t)m * i] = acc;
      }
    free(V);
  }
}

/* ------------------------------------------------------------------------ */
/* A16 get_dij: get_dij.f90:13-31,100-155                                     */
/*   D = D0 + D_H(rho) + D_xc(rho) + Dhat[v_ks - v_xc];  D_H_ij = sum_kl E_ijkl rho_kl ;   */
/*   Dhat_ij = dv sum_g (v_ks - v_xc)(r_g) sum_lm q_ij^lm g_lm(r_g): get_dij   */
/*   passes vks and vxc to pawdij, which builds Dhat on vtrial - vxc when the  */
/*   compensation charge is not in the XC density (usexcnhat = 0,            */
/*   1_libpaw_mod.f90:49; libpaw/4_m_pawdij.F90:375-385)                      */
/*   lower triangle mirrored and clamped at dij_max (:140-150)                 */
/* ------------------------------------------------------------------------ */
void orc_dij(orc_ctx *c, int set) {
  double *dxc = NULL;
  if (c->oxc) {
    dxc = (double *)calloc(c->nd ? c->nd : 1, sizeof(double));
    orc_onsite_xc(c, c->rhoij[set], dxc);
  }
  for (int a = 0; a < c->natom; a++) {
    int m = c->ms[a], L = c->nlm[a], ng = c->ngrid[a];
    const double *R = c->rhoij[set] + c->doff[a];
    const double *Q = c->qijlm + c->qoff[a];
    const double *G = c->g3d + c->g3off[a];
    const double *E = c->eijkl + c->eoff[a];
    const double *D0 = c->dij0 + c->doff[a];
    const int *lg = c->local_grid + 3 * c->goff[a];
    double prod[64];
    for (int l = 0; l < L; l++) {
      double acc = 0;
      for (int ig = 0; ig < ng; ig++) {
        size_t gi = (lg[3 * ig] - 1) + (size_t)c->nx * ((lg[3 * ig + 1] - 1) + (size_t)c->ny * (lg[3 * ig + 2] - 1));
        acc += (c->vks[set][gi] - c->vxc[set][gi]) * G[ig + (size_t)ng * l];
      }
      prod[l] = acc * c->dv;
    }
    double *D = c->dij[set] + c->doff[a];
    for (int j = 0; j < m; j++)
      for (int i = j; i < m; i++) {
        double d = D0[i + (size_t)m * j];
        for (int l2 = 0; l2 < m; l2++)
          for (int k = 0; k < m; k++)
            d += E[i + (size_t)m * (j + (size_t)m * (k + (size_t)m * l2))] * R[k + (size_t)m * l2];
        for (int l = 0; l < L; l++) d += prod[l] * Q[l + (size_t)L * (i + (size_t)m * j)];
        if (dxc) d += dxc[c->doff[a] + i + (size_t)m * j];
        double mx = c->sys.dij_max;
        if (mx > 0 && fabs(d) > mx) d = d / fabs(d) * mx; /* :144 */
        D[i + (size_t)m * j] = d;
        D[j + (size_t)m * i] = d;
      }
  }
  free(dxc);
}

/* ------------------------------------------------------------------------ */
/* A7 ncpaw_make_hamiltonian_tddft_{unpert,pert}: ncpaw_make_hamiltonian.f90:213-281 */
/* ------------------------------------------------------------------------ */
void orc_rebuild(orc_ctx *c, int set, const cplx *psibar, int norb) {
  cplx *t = (cplx *)malloc(sizeof(cplx) * c->nn * (size_t)norb);
  orc_sn_phi_batch(c, -0.5, psibar, t, norb); /* :119-122 */
  orc_rhoij(c, set, t, norb);                  /* :125 */
  orc_density(c, set, t, norb);                /* :126 */
  orc_nhat(c, set);                            /* :127 */
  orc_vks(c, set);                             /* :128 */
  orc_dij(c, set);                             /* :129 */
  free(t);
}

/* ------------------------------------------------------------------------ */
/* A18 excite_psi_bar_pert: tddft_excite.f90:8-15                             */
/* ------------------------------------------------------------------------ */
static double rcoord(int i, int n, double d) { return (double)(i - n / 2) * d; } /* (ix-1-nx/2)*dx */

void orc_excite(const orc_ctx *c, int ipol, double gamma, const cplx *psi, cplx *pp, int norb) {
  for (int b = 0; b < norb; b++)
    for (int iz = 0; iz < c->nz; iz++)
      for (int iy = 0; iy < c->ny; iy++)
        for (int ix = 0; ix < c->nx; ix++) {
          double r[3] = {rcoord(ix, c->nx, c->sys.dx), rcoord(iy, c->ny, c->sys.dy), rcoord(iz, c->nz, c->sys.dz)};
          double ph = -gamma * r[ipol - 1];
          size_t i = (size_t)b * c->nn + ix + (size_t)c->nx * (iy + (size_t)c->ny * iz);
          pp[i] = psi[i] * (cos(ph) + sin(ph) * I);
        }
}

/* ------------------------------------------------------------------------ */
/* A19 plot_dip: tddft_plot.f90:30-57,116-150 (h_type = 1: psi_bar directly)  */
/* ------------------------------------------------------------------------ */
void orc_dipole(const orc_ctx *c, const cplx *p, const cplx *pp, int norb, double gamma, double *dip,
                double *dip_pert, double *d_dip) {
  for (int k = 0; k < 3; k++) dip[k] = dip_pert[k] = 0;
  size_t i = 0;
  for (int iz = 0; iz < c->nz; iz++)
    for (int iy = 0; iy < c->ny; iy++)
      for (int ix = 0; ix < c->nx; ix++, i++) {
        double r[3] = {rcoord(ix, c->nx, c->sys.dx), rcoord(iy, c->ny, c->sys.dy), rcoord(iz, c->nz, c->sys.dz)};
        double rho = 0, rhop = 0;
        for (int b = 0; b < norb; b++) {
          cplx z = p[(size_t)b * c->nn + i], w = pp[(size_t)b * c->nn + i];
          rho += creal(z) * creal(z) + cimag(z) * cimag(z);
          rhop += creal(w) * creal(w) + cimag(w) * cimag(w);
        }
        rho *= 2.0;
        rhop *= 2.0;
        for (int k = 0; k < 3; k++) {
          dip[k] += c->dv * r[k] * rho;
          dip_pert[k] += c->dv * r[k] * rhop;
        }
      }
  for (int k = 0; k < 3; k++) d_dip[k] = (dip_pert[k] - dip[k]) / gamma; /* :57 */
}

/* ------------------------------------------------------------------------ */
/* A6 rk4_prop_shs: rk4.f90:15-102 for one set                                */
/* ------------------------------------------------------------------------ */
static void rk4_set(orc_ctx *c, int set, cplx *p, int norb, double dt) {
  size_t nn = c->nn, tot = nn * (size_t)norb;
  cplx *p2 = (cplx *)malloc(sizeof(cplx) * tot), *k1 = (cplx *)malloc(sizeof(cplx) * tot),
       *k2 = (cplx *)malloc(sizeof(cplx) * tot), *k4 = (cplx *)malloc(sizeof(cplx) * tot),
       *y = (cplx *)malloc(sizeof(cplx) * tot);
  double *nrm0 = (double *)malloc(sizeof(double) * norb);
  memcpy(p2, p, sizeof(cplx) * tot); /* :15 */
  for (int b = 0; b < norb; b++) {   /* norm0 :81-90 */
    double s = 0;
    for (size_t i = 0; i < nn; i++) { cplx z = p2[(size_t)b * nn + i]; s += creal(z) * creal(z) + cimag(z) * cimag(z); }
    nrm0[b] = sqrt(c->dv * s);
  }
  /* stage(pin, k, dtst, last): k = -i shs(pin); y = p2 + dtst k; rebuild(y)  :35-56 */
  cplx *ks[4] = {k1, k2, k4, k4};
  double dts[4] = {dt / 2.0, dt / 2.0, dt, dt};
  for (int st = 0; st < 4; st++) {
    const cplx *pin = (st == 0) ? p2 : y;
    cplx *k = ks[st];
    if (st == 3) {
      for (size_t i = 0; i < tot; i++) k2[i] = k2[i] + k4[i]; /* :20 k2 = k2 + k3 */
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int b = 0; b < norb; b++) orc_shs(c, set, pin + (size_t)b * nn, k + (size_t)b * nn);
    for (size_t i = 0; i < tot; i++) k[i] = -I * k[i];
    if (st < 3) {
      for (size_t i = 0; i < tot; i++) y[i] = p2[i] + dts[st] * k[i];
      orc_rebuild(c, set, y, norb);
    }
  }
  for (size_t i = 0; i < tot; i++) p[i] = p2[i] + dt / 6.0 * (k1[i] + 2.0 * k2[i] + k4[i]); /* :22 */
  for (int b = 0; b < norb; b++) { /* norm1 :92-102 */
    double s = 0;
    for (size_t i = 0; i < nn; i++) { cplx z = p[(size_t)b * nn + i]; s += creal(z) * creal(z) + cimag(z) * cimag(z); }
    double n1 = sqrt(c->dv * s);
    for (size_t i = 0; i < nn; i++) p[(size_t)b * nn + i] *= nrm0[b] / n1;
  }
  free(p2); free(k1); free(k2); free(k4); free(y); free(nrm0);
}

void orc_rk4_prop_shs(orc_ctx *c, cplx *p, cplx *pp, int norb, double dt) {
  rk4_set(c, 0, p, norb, dt);  /* :15-23 */
  rk4_set(c, 1, pp, norb, dt); /* :25-33 */
}

/* opaw_tddft loop body (tddft.f90:67-91, dyn = 3): rebuild both sets, propagate, dipole */
void orc_tddft_steps(orc_ctx *c, cplx *p, cplx *pp, int norb, int nsteps, double dt, double gamma,
                     double *d_dip_out) {
  for (int it = 0; it < nsteps; it++) {
    orc_rebuild(c, 0, p, norb); /* ncpaw_make_hamiltonian_tddft :118-167 */
    orc_rebuild(c, 1, pp, norb);
    orc_rk4_prop_shs(c, p, pp, norb, dt);
    double dip[3], dipp[3], dd[3];
    orc_dipole(c, p, pp, norb, gamma, dip, dipp, dd);
    if (d_dip_out) for (int k = 0; k < 3; k++) d_dip_out[3 * it + k] = dd[k];
  }
}

int orc_nthreads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
