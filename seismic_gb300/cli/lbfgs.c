/* lbfgs.c - L_BFGS.x: one step of the out-of-core limited-memory BFGS
 * (progs/inversion/L_BFGS.f90:1-103 with libs/libnlinv) over libswave.
 *
 *   L_BFGS.x Model=mod.H Gradient=grad.H Function=fct.H
 *            [Initial_Model=init.H Gradient_Weight=w.H]
 *            lbfgs_type=0|1 bound_type=1|2 stp1_opt=0|1 step_init= xmin= xmax=
 *
 * Each invocation makes one reverse-communication call of LBFGSOLD
 * (lbfgs_type 0, the default) or LBFGSOC (lbfgs_type 1: the model's nparams
 * blocks clipped to xmin[j], xmax[j]) at the model, objective and gradient
 * given, and writes the next model to evaluate over the Model dataset.
 * Everything the solver keeps between calls travels through files in the
 * working directory, as in the reference (nlinv_read_array_params.f90:
 * 139-155): it reads Iflag.dat, Info.dat (text), Diag.dat, WorkArray.dat
 * (Fortran unformatted sequential records of doubles), LbfgsDat.dat and
 * McsrchDat.dat (list-directed text of the saved scalars) when they exist,
 * and writes the same files with the suffix Out (IflagOut.dat, ...); the
 * caller renames them before the next invocation.  log.dat and
 * bfgsiter.dat receive a log.  The solver's vectors run on the GPU in FP64
 * (sw_lbfgs_oc_step).
 */
#include <ctype.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "swcli.h"

/* ---- Fortran unformatted sequential records (4-byte length markers;
 * records above 2^31 - 1 bytes split into subrecords whose leading marker
 * is negative while the record continues, and whose trailing marker is
 * negative for every subrecord but the first). --------------------------- */
static const int64_t kSubMax = 2147483639;

static int write_record(const char *path, const void *data, int64_t bytes) {
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  const char *p = (const char *)data;
  int64_t left = bytes, done = 0;
  int first = 1;
  do {
    const int64_t chunk = left > kSubMax ? kSubMax : left;
    const int32_t len = (int32_t)chunk;
    const int32_t lead = left > kSubMax ? -len : len;
    const int32_t trail = first ? len : -len;
    if (fwrite(&lead, 4, 1, f) != 1 || (chunk && fwrite(p + done, 1, (size_t)chunk, f) != (size_t)chunk) ||
        fwrite(&trail, 4, 1, f) != 1) {
      fclose(f);
      return -1;
    }
    done += chunk;
    left -= chunk;
    first = 0;
  } while (left > 0);
  return fclose(f);
}

static int read_record(const char *path, void *data, int64_t bytes) {
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  char *p = (char *)data;
  int64_t done = 0;
  for (;;) {
    int32_t lead, trail;
    if (fread(&lead, 4, 1, f) != 1) break;
    const int64_t chunk = lead < 0 ? -(int64_t)lead : lead;
    if (done + chunk > bytes || (chunk && fread(p + done, 1, (size_t)chunk, f) != (size_t)chunk) ||
        fread(&trail, 4, 1, f) != 1)
      break;
    done += chunk;
    if (lead >= 0) {
      fclose(f);
      return done == bytes ? 0 : -1;
    }
  }
  fclose(f);
  return -1;
}

/* ---- List-directed text of the saved scalars ---------------------------- */
typedef struct field {
  const char *name;
  int is_int;
  size_t off;
} field;

#define FD(x) {#x, 0, offsetof(sw_lbfgs_oc_state, x)}
#define FI(x) {#x, 1, offsetof(sw_lbfgs_oc_state, x)}
/* LbfgsDat.dat lines (nlinv_lbfgs.f:277-281). */
static const field kLbfgsLines[5][9] = {
    {FD(gtol), FD(one), FD(zero), FD(gnorm), FD(stp1), FD(ftol), FD(stpmin)},
    {FD(stpmax), FD(stp), FD(ys), FD(yy), FD(sq), FD(yr), FD(beta), FD(xnorm)},
    {FI(mp), FI(lp), FI(iter), FI(nfun), FI(point), FI(ispt), FI(iypt), FI(maxfev), FI(info)},
    {FI(bound), FI(npt), FI(cp), FI(i), FI(nfev), FI(inmc), FI(iycn), FI(iscn)},
    {FI(finish)}};
/* McsrchDat.dat lines (nlinv_lbfgs.f:725-730). */
static const field kMcsrchLines[5][9] = {
    {FI(infoc), FI(j)},
    {FI(brackt), FI(stage1)},
    {FD(dg), FD(dgm), FD(dginit), FD(dgtest), FD(dgx), FD(dgxm), FD(dgy), FD(dgym)},
    {FD(finit), FD(ftest1), FD(fm), FD(fx), FD(fxm), FD(fy), FD(fym), FD(stx), FD(sty)},
    {FD(stmin), FD(stmax), FD(width), FD(width1)}};
/* Fields written as Fortran logicals. */
static int is_logical(const char *n) {
  return !strcmp(n, "finish") || !strcmp(n, "brackt") || !strcmp(n, "stage1");
}

static int write_scalars(const char *path, const sw_lbfgs_oc_state *st, const field (*lines)[9]) {
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  for (int l = 0; l < 5; ++l) {
    for (int k = 0; k < 9 && lines[l][k].name; ++k) {
      const char *base = (const char *)st + lines[l][k].off;
      if (lines[l][k].is_int) {
        const int v = *(const int *)base;
        if (is_logical(lines[l][k].name)) fprintf(f, " %s", v ? "T" : "F");
        else fprintf(f, " %d", v);
      } else {
        fprintf(f, " %.17g", *(const double *)base);
      }
    }
    fputc('\n', f);
  }
  return fclose(f);
}

/* Reads the values in order (list-directed: separated by blanks, commas or
 * line ends; logicals T / F / .TRUE. / .FALSE.). */
static int read_scalars(const char *path, sw_lbfgs_oc_state *st, const field (*lines)[9]) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  char tok[128];
  int rc = 0;
  for (int l = 0; l < 5 && !rc; ++l)
    for (int k = 0; k < 9 && lines[l][k].name && !rc; ++k) {
      if (fscanf(f, " %127[^ \t\r\n,]%*[ ,]", tok) < 1) {
        rc = -1;
        break;
      }
      char *base = (char *)st + lines[l][k].off;
      if (lines[l][k].is_int) {
        if (is_logical(lines[l][k].name)) {
          const char *t = tok[0] == '.' ? tok + 1 : tok;
          *(int *)base = toupper((unsigned char)t[0]) == 'T';
        } else {
          *(int *)base = atoi(tok);
        }
      } else {
        for (char *q = tok; *q; ++q)
          if (*q == 'D' || *q == 'd') *q = 'e';   /* Fortran exponent letter */
        *(double *)base = strtod(tok, NULL);
      }
    }
  fclose(f);
  return rc;
}

static int read_int_file(const char *path, int *v) {
  FILE *f = fopen(path, "r");
  if (!f) return 0;
  const int ok = fscanf(f, "%d", v) == 1;
  fclose(f);
  return ok ? 1 : -1;
}

static void write_int_file(const char *path, int v) {
  FILE *f = fopen(path, "w");
  if (!f || fprintf(f, "%2d\n", v) < 0 || fclose(f)) cli_fail("cannot write %s", path);
}

static int file_exists(const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) return 0;
  fclose(f);
  return 1;
}

/* A dataset's samples and axes (read_sepfile, nlinv_io.f90:29-53). */
typedef struct dataset {
  int n[4], ndim;
  float o[4], d[4];
  size_t size;
  float *a;
} dataset;

static void read_dataset(const char *tag, dataset *ds) {
  sep_file *f = sep_open_in(tag);
  if (!f) cli_fail("%s file is missing: %s", tag, sep_error());
  ds->ndim = 1;
  ds->size = 1;
  for (int i = 0; i < 4; ++i) {
    char key[8];
    ds->n[i] = 1;
    ds->o[i] = 0.f;
    ds->d[i] = 1.f;
    snprintf(key, sizeof key, "n%d", i + 1);
    sep_hdr_int(f, key, &ds->n[i]);
    snprintf(key, sizeof key, "o%d", i + 1);
    sep_hdr_float(f, key, &ds->o[i]);
    snprintf(key, sizeof key, "d%d", i + 1);
    sep_hdr_float(f, key, &ds->d[i]);
    if (ds->n[i] < 1) cli_fail("%s: n%d = %d", tag, i + 1, ds->n[i]);
    if (ds->n[i] > 1) ds->ndim = i + 1;
    ds->size *= (size_t)ds->n[i];
  }
  ds->a = (float *)malloc(ds->size * sizeof(float));
  if (!ds->a || sep_read(f, ds->a, ds->size)) cli_fail("cannot read %s: %s", tag, sep_error());
  sep_close(f);
}

static void same_shape(const dataset *a, const dataset *b, const char *what) {
  for (int i = 0; i < 4; ++i)
    if (a->n[i] != b->n[i]) cli_fail("%s have different sizes, exit now", what);
}

/* xmin= / xmax=: nparams comma-separated values, 0 where absent. */
static void read_list(const char *name, int np, double *out) {
  char buf[1024] = "";
  for (int j = 0; j < np; ++j) out[j] = 0.0;
  if (sep_par_str(name, buf, sizeof buf) <= 0) return;
  char *p = buf;
  for (int j = 0; j < np && *p; ++j) {
    out[j] = strtod(p, &p);
    while (*p == ',' || *p == ' ') ++p;
  }
}

int main(int argc, char **argv) {
  if (sep_init(argc, argv)) cli_fail("%s", sep_error());
  FILE *lg = fopen("log.dat", "a"), *it = fopen("bfgsiter.dat", "a");
  if (!lg || !it) cli_fail("cannot open log.dat / bfgsiter.dat");
  int lbfgs_type = 0, bound_type = 1, stp1_opt = 1;
  float step_init = 999999.f;
  sep_par_int("lbfgs_type", &lbfgs_type);
  sep_par_int("bound_type", &bound_type);
  sep_par_int("stp1_opt", &stp1_opt);
  sep_par_float("step_init", &step_init);
  fprintf(stderr, "INFO: lbfgs_type = %d, bound_type = %d, stp1_opt = %d\n", lbfgs_type,
          bound_type, stp1_opt);
  /* lbfgs_setup_sepfile (nlinv_read_array_params.f90:11-118). */
  dataset mod, fct, gdt, modi, wgh;
  read_dataset("Model", &mod);
  read_dataset("Function", &fct);
  read_dataset("Gradient", &gdt);
  if (lbfgs_type == 1) {
    read_dataset("Initial_Model", &modi);
    same_shape(&mod, &modi, "Model and initial model");
    if (sep_exist("Gradient_Weight")) {
      read_dataset("Gradient_Weight", &wgh);
      same_shape(&gdt, &wgh, "Gradient and Gradient weight");
      free(wgh.a);
    }
    free(modi.a);
  }
  same_shape(&gdt, &mod, "Gradient and Model");
  /* lbfgs_setup (:120-271): the last axis is the parameter axis when the
   * gradient has 3 axes and n3 < 5, or 4 axes. */
  const int n = (int)gdt.size;
  int nparams = 1;
  if (gdt.ndim == 3 && gdt.n[2] < 5) nparams = gdt.n[2];
  else if (gdt.ndim == 4) nparams = gdt.n[3];
  fprintf(lg, " We are inverting for %d parameters\n", nparams);
  double *xmin = (double *)calloc((size_t)nparams, sizeof(double));
  double *xmax = (double *)calloc((size_t)nparams, sizeof(double));
  if (!xmin || !xmax) cli_fail("out of host memory");
  if (lbfgs_type == 1) {
    read_list("xmin", nparams, xmin);
    read_list("xmax", nparams, xmax);
  }
  const int m = 5;
  const size_t nwork = (size_t)n * (2 * m + 1) + 2 * m;
  int iflag = 0, myinfo = 0;
  if (read_int_file("Iflag.dat", &iflag) < 0) cli_fail("cannot read Iflag.dat");
  if (read_int_file("Info.dat", &myinfo) < 0) cli_fail("cannot read Info.dat");
  fprintf(lg, " Reading iflag= %d\n Reading myinfo= %d\n", iflag, myinfo);
  double *w = (double *)calloc(nwork, sizeof(double));
  double *diag = (double *)calloc((size_t)n, sizeof(double));
  double *x = (double *)malloc((size_t)n * sizeof(double));
  double *g = (double *)malloc((size_t)n * sizeof(double));
  if (!w || !diag || !x || !g) cli_fail("out of host memory");
  sw_lbfgs_oc_state st;
  memset(&st, 0, sizeof st);
  if (iflag != 0) {
    if (read_record("Diag.dat", diag, (int64_t)n * 8) ||
        read_record("WorkArray.dat", w, (int64_t)nwork * 8))
      cli_fail("cannot read Diag.dat / WorkArray.dat for n = %d", n);
    if (read_scalars("LbfgsDat.dat", &st, kLbfgsLines)) cli_fail("cannot read LbfgsDat.dat");
    if (st.info != 0 && file_exists("McsrchDat.dat") &&
        read_scalars("McsrchDat.dat", &st, kMcsrchLines))
      cli_fail("cannot read McsrchDat.dat");
  }
  for (int i = 0; i < n; ++i) {
    x[i] = mod.a[i];
    g[i] = gdt.a[i];
  }
  const double f = fct.a[0];
  sw_lbfgs_oc_desc d;
  memset(&d, 0, sizeof d);
  d.n = n;
  d.m = m;
  d.nparam = nparams;
  d.xmin = xmin;
  d.xmax = xmax;
  d.lbfgs_type = lbfgs_type;
  d.bound_type = bound_type;
  d.stp1_opt = stp1_opt;
  d.step_init = (double)step_init;
  d.eps = 1.0e-20;
  d.xtol = 2.220446049250313e-16;
  sw_ctx *ctx = cli_context();
  cli_check(ctx, sw_lbfgs_oc_step(ctx, &d, x, f, g, w, diag, &st, &iflag, &myinfo),
            "sw_lbfgs_oc_step");
  sw_ctx_destroy(ctx);
  fprintf(it, " iter %d nfun %d f %.10g stp %.10g iflag %d\n", st.iter, st.nfun, f, st.stp,
          iflag);
  if (write_scalars("LbfgsDatOut.dat", &st, kLbfgsLines) ||
      write_scalars("McsrchDatOut.dat", &st, kMcsrchLines))
    cli_fail("cannot write the solver state");
  fprintf(lg, " Writing working array\n");
  if (write_record("WorkArrayOut.dat", w, (int64_t)nwork * 8)) cli_fail("cannot write WorkArrayOut.dat");
  fprintf(lg, " Writing diag\n");
  if (write_record("DiagOut.dat", diag, (int64_t)n * 8)) cli_fail("cannot write DiagOut.dat");
  fprintf(lg, " Writing iflag= %d\n", iflag);
  write_int_file("IflagOut.dat", iflag);
  fprintf(lg, " Writing myinfo= %d\n", myinfo);
  write_int_file("InfoOut.dat", myinfo);
  /* The next model over the Model dataset (write_sepfile, nlinv_io.f90:55-68). */
  for (int i = 0; i < n; ++i) mod.a[i] = (float)x[i];
  sep_file *fo = sep_open_out("Model");
  if (!fo) cli_fail("%s", sep_error());
  for (int i = 0; i < 4; ++i) {
    char key[8];
    snprintf(key, sizeof key, "n%d", i + 1);
    sep_put_int(fo, key, mod.n[i]);
    snprintf(key, sizeof key, "o%d", i + 1);
    sep_put_float(fo, key, mod.o[i]);
    snprintf(key, sizeof key, "d%d", i + 1);
    sep_put_float(fo, key, mod.d[i]);
  }
  if (sep_write(fo, mod.a, mod.size) || sep_close(fo)) cli_fail("cannot write Model: %s", sep_error());
  fclose(lg);
  fclose(it);
  free(w); free(diag); free(x); free(g); free(xmin); free(xmax);
  free(mod.a); free(fct.a); free(gdt.a);
  sep_finish();
  return 0;
}
