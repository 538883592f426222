/* swcli.c - reading and writing steps shared by the command-line programs
 * (see swcli.h). */
#include "swcli.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void cli_fail(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  fprintf(stderr, "ERROR: ");
  vfprintf(stderr, fmt, ap);
  fprintf(stderr, "\n");
  va_end(ap);
  exit(1);
}

static void *xmalloc(size_t n) {
  void *p = malloc(n ? n : 1);
  if (!p) cli_fail("out of host memory (%zu bytes)", n);
  return p;
}

static void par_int(const char *name, int *v, int def) {
  *v = def;
  if (sep_par_int(name, v) < 0) cli_fail("parameter %s is not an integer", name);
}
static void par_float(const char *name, float *v, float def) {
  *v = def;
  if (sep_par_float(name, v) < 0) cli_fail("parameter %s is not a number", name);
}
static void par_bool(const char *name, int *v, int def) {
  *v = def;
  if (sep_par_bool(name, v) < 0) cli_fail("parameter %s is not a logical (y/n, 1/0)", name);
}

void cli_read_params(cli_par *p) {
  memset(p, 0, sizeof(*p));
  sw_genpar *g = &p->g;
  par_float("fmax", &g->fmax, 30.f);
  par_int("ntaper", &g->ntaper, 20);
  par_int("snapi", &g->snapi, 4);
  par_float("aperture_x", &p->aperture_x, 0.f);
  par_float("aperture_y", &p->aperture_y, 0.f);
  par_int("num_threads", &p->nthreads, 4);
  par_int("lsinc", &g->lsinc, 7);
  par_float("maxsize", &p->max_memory, 16.f);
  par_int("rec_type", &g->rec_type, 0);
  par_int("shot_type", &g->shot_type, 0);
  par_int("surf_type", &g->surf_type, 0);
  par_bool("twoD", &g->twoD, 0);
  par_bool("withRho", &p->withRho, 0);
  par_bool("LSRTM", &p->LSRTM, 0);
  par_bool("Born", &p->Born, 0);
  par_bool("verb", &p->verbose, 1);
  snprintf(p->task, sizeof(p->task), "MOD");
  sep_par_str("Task", p->task, sizeof(p->task));
  if (p->LSRTM) par_bool("CHEAPLSRTM", &p->CHEAPLSRTM, 0);
  par_bool("write_forward_wavefield", &p->WriteFwdWvfld, 0);
  if (p->verbose) {
    fprintf(stderr, "INFO: task=%s fmax=%g ntaper=%d snapi=%d aperture_x=%g aperture_y=%g\n",
            p->task, (double)g->fmax, g->ntaper, g->snapi, (double)p->aperture_x,
            (double)p->aperture_y);
    fprintf(stderr, "INFO: lsinc=%d twoD=%d LSRTM=%d Born=%d\n", g->lsinc, g->twoD, p->LSRTM,
            p->Born);
  }
}

float *cli_read_source(cli_par *p) {
  sep_file *f = sep_open_in("in");
  if (!f) cli_fail("%s", sep_error());
  int nt = 0;
  float dt = 0.f, ot = 0.f;
  if (sep_hdr_int(f, "n1", &nt) != 1 || nt < 1) cli_fail("wavelet header needs n1");
  if (sep_hdr_float(f, "d1", &dt) != 1 || !(dt > 0.f)) cli_fail("wavelet header needs d1");
  sep_hdr_float(f, "o1", &ot);
  float *w = (float *)xmalloc((size_t)nt * 4);
  if (sep_read(f, w, (size_t)nt)) cli_fail("%s", sep_error());
  sep_close(f);
  p->g.nt = nt;
  p->g.dt = dt;
  if (p->Born || p->LSRTM) sw_born_wavelet(w, nt, dt);
  if (p->withRho) sw_rho_wavelet(w, nt, p->g.lsinc);
  return w;
}

float *cli_read_traces(int nt, int *ntr, float *ot) {
  if (!sep_exist("traces")) cli_fail("need traces file");
  sep_file *f = sep_open_in("traces");
  if (!f) cli_fail("%s", sep_error());
  int n1 = 0, n2 = 0;
  if (sep_hdr_int(f, "n1", &n1) != 1) cli_fail("traces header needs n1");
  if (sep_hdr_int(f, "n2", &n2) != 1 || n2 < 1) cli_fail("traces header needs n2");
  if (n1 != nt) cli_fail("nt traces and sources are different, exit now");
  if (ot) {
    *ot = 0.f;
    sep_hdr_float(f, "o1", ot);
  }
  float *t = (float *)xmalloc((size_t)n1 * n2 * 4);
  if (sep_read(f, t, (size_t)n1 * n2)) cli_fail("%s", sep_error());
  sep_close(f);
  *ntr = n2;
  return t;
}

float *cli_read_coords(int ntr, float sou[3]) {
  const char *names[6] = {"keygx", "keysx", "keygy", "keysy", "keyselev", "keygelev"};
  int idx[6];
  for (int k = 0; k < 6; ++k)
    if (sep_par_int(names[k], &idx[k]) != 1) cli_fail("need %s", names[k]);
  if (!sep_exist("coordfile")) cli_fail("need coordfile");
  sep_file *f = sep_open_in("coordfile");
  if (!f) cli_fail("%s", sep_error());
  int nkeys = 0, n2 = 0;
  if (sep_hdr_int(f, "n1", &nkeys) != 1 || nkeys < 1) cli_fail("coordfile header needs n1");
  if (sep_hdr_int(f, "n2", &n2) != 1) cli_fail("coordfile header needs n2");
  if (n2 != ntr) cli_fail("size datavec ne number of traces in coordfiles, exit");
  for (int k = 0; k < 6; ++k)
    if (idx[k] < 1 || idx[k] > nkeys) cli_fail("%s=%d is outside 1..%d", names[k], idx[k], nkeys);
  float *keys = (float *)xmalloc((size_t)nkeys * 4);
  float *rec = (float *)xmalloc((size_t)ntr * 3 * 4);
  for (int i = 0; i < ntr; ++i) {
    if (sep_read(f, keys, (size_t)nkeys)) cli_fail("%s", sep_error());
    rec[3 * i + 0] = keys[idx[5] - 1];
    rec[3 * i + 1] = keys[idx[0] - 1];
    rec[3 * i + 2] = keys[idx[2] - 1];
  }
  sou[0] = keys[idx[4] - 1];
  sou[1] = keys[idx[1] - 1];
  sou[2] = keys[idx[3] - 1];
  sep_close(f);
  free(keys);
  fprintf(stderr, "INFO: source z=%g x=%g y=%g, %d receivers\n", (double)sou[0], (double)sou[1],
          (double)sou[2], ntr);
  return rec;
}

float *cli_read_model(cli_par *p, const char *tag) {
  if (!sep_exist(tag)) cli_fail("need %s file", tag);
  sep_file *f = sep_open_in(tag);
  if (!f) cli_fail("%s", sep_error());
  int n[3] = {1, 1, 1};
  float o[3] = {0.f, 0.f, 0.f}, d[3] = {1.f, 1.f, 1.f};
  const int naxes = p->g.twoD ? 2 : 3;
  for (int a = 0; a < naxes; ++a) {
    char kn[4] = {'n', (char)('1' + a), 0}, ko[4] = {'o', (char)('1' + a), 0},
         kd[4] = {'d', (char)('1' + a), 0};
    if (sep_hdr_int(f, kn, &n[a]) != 1 || n[a] < 1) cli_fail("%s: need %s", tag, kn);
    if (sep_hdr_float(f, ko, &o[a]) != 1) cli_fail("%s: need %s", tag, ko);
    if (sep_hdr_float(f, kd, &d[a]) != 1 || !(d[a] > 0.f)) cli_fail("%s: need %s", tag, kd);
  }
  sw_genpar *g = &p->g;
  if (g->nz == 0) {
    g->nz = n[0];
    g->nx = n[1];
    g->ny = n[2];
    g->oz = o[0];
    g->ox = o[1];
    g->oy = o[2];
    g->dz = d[0];
    g->dx = d[1];
    g->dy = d[2];
  } else {
    const int nn[3] = {g->nz, g->nx, g->ny};
    const float oo[3] = {g->oz, g->ox, g->oy}, dd[3] = {g->dz, g->dx, g->dy};
    for (int a = 0; a < naxes; ++a) {
      if (n[a] != nn[a]) cli_fail("vel %s not consistent with n%d", tag, a + 1);
      if (o[a] != oo[a]) cli_fail("vel %s not consistent with o%d", tag, a + 1);
      if (d[a] != dd[a]) cli_fail("vel %s not consistent with d%d", tag, a + 1);
    }
  }
  const size_t cnt = (size_t)n[0] * n[1] * n[2];
  float *v = (float *)xmalloc(cnt * 4);
  if (sep_read(f, v, cnt)) cli_fail("%s", sep_error());
  sep_close(f);
  return v;
}

void cli_shot_window(const cli_par *p, const float sou[3], int ntr, const float *rec,
                     sw_window *w, sw_genpar *gw) {
  const sw_genpar *m = &p->g;
  if (sw_shot_window(m, p->aperture_x, p->aperture_y, sou, ntr, rec, w) != SW_OK)
    cli_fail("degenerate source/receiver window");
  const float xend = m->ox + (float)(m->nx - 1) * m->dx;
  const float yend = m->oy + (float)(m->ny - 1) * m->dy;
  /* The check sees the patch's y origin before 2D resets it to oy. */
  float oyw = w->oyw;
  if (m->twoD) {
    float gy1 = rec[2], gyn = rec[2];
    for (int i = 1; i < ntr; ++i) {
      gy1 = rec[3 * i + 2] < gy1 ? rec[3 * i + 2] : gy1;
      gyn = rec[3 * i + 2] > gyn ? rec[3 * i + 2] : gyn;
    }
    const float my1 = (gy1 + sou[2]) / 2, myn = (gyn + sou[2]) / 2;
    const float cy = my1 + fabsf(myn - my1) / 2;
    const float miny = sou[2] < gy1 ? sou[2] : gy1;
    oyw = miny < cy - p->aperture_y / 2 ? miny : cy - p->aperture_y / 2;
  }
  int nout = 0;
  if (w->oxw < m->ox || w->oxw > xend) ++nout;
  if (w->endx < m->ox || w->endx > xend) ++nout;
  if (oyw < m->oy || oyw > yend) ++nout;
  if (w->endy < m->oy || w->endy > yend) ++nout;
  if (w->oxw < m->ox && w->endx > xend) --nout;
  if (oyw < m->oy && w->endy > yend) --nout;
  if (nout == 4)
    cli_fail("the source/receiver patch, with aperture, is outside velocity model "
             "(oxw=%g endx=%g oyw=%g endy=%g)",
             (double)w->oxw, (double)w->endx, (double)oyw, (double)w->endy);
  *gw = *m;
  gw->nx = w->nxw;
  gw->ny = w->nyw;
  gw->ox = w->oxw;
  gw->oy = w->oyw;
  fprintf(stderr, "INFO: window nz=%d nx=%d ny=%d ox=%g oy=%g\n", gw->nz, gw->nx, gw->ny,
          (double)gw->ox, (double)gw->oy);
}

static void write_or_fail(sep_file *f, const float *v, size_t n) {
  if (sep_write(f, v, n)) cli_fail("%s", sep_error());
}

void cli_write_image(const cli_par *p, const char *tag, const float *image, const float *illum) {
  const sw_genpar *g = &p->g;
  sep_file *f = sep_open_out(tag);
  if (!f) cli_fail("%s", sep_error());
  const size_t n = (size_t)g->nz * g->nx * g->ny;
  write_or_fail(f, image, n);
  write_or_fail(f, illum, n);
  sep_put_int(f, "n1", g->nz);
  sep_put_int(f, "n2", g->nx);
  sep_put_float(f, "d1", g->dz);
  sep_put_float(f, "d2", g->dx);
  sep_put_float(f, "o1", g->oz);
  sep_put_float(f, "o2", g->ox);
  if (g->twoD) {
    sep_put_int(f, "n3", 2);
  } else {
    sep_put_int(f, "n3", g->ny);
    sep_put_float(f, "d3", g->dy);
    sep_put_float(f, "o3", g->oy);
    sep_put_int(f, "n4", 2);
  }
  if (sep_close(f)) cli_fail("%s", sep_error());
}

void cli_write_traces(const cli_par *p, const char *tag, int ntr, const float *data) {
  sep_file *f = sep_open_out(tag);
  if (!f) cli_fail("%s", sep_error());
  write_or_fail(f, data, (size_t)ntr * p->g.nt);
  sep_put_int(f, "n1", p->g.nt);
  sep_put_int(f, "n2", ntr);
  sep_put_float(f, "d1", p->g.dt);
  sep_put_float(f, "d2", 1.f);
  sep_put_float(f, "o1", 0.f);
  sep_put_float(f, "o2", 0.f);
  if (sep_close(f)) cli_fail("%s", sep_error());
}

sw_ctx *cli_context(void) {
  sw_ctx *c = NULL;
  if (sw_ctx_create(0, &c) != SW_OK || !c)
    cli_fail("cannot create a swave context on CUDA device 0 (is a GPU visible?)");
  return c;
}

void cli_check(sw_ctx *ctx, int status, const char *what) {
  if (status != SW_OK) cli_fail("%s failed (%d): %s", what, status, sw_last_error(ctx));
}
