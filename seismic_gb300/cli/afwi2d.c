/* 2DAFWI.x - multi-shot acoustic modelling and migration over a survey
 * (progs/afwi/2DAFWI.f90).  The wavelet comes from stdin= (or standard
 * input), the model from vel=, and the survey from coordfile= (n1 keys by
 * n2 traces); consecutive traces with the same (sx, sy) form one shot
 * gather (readgathercoords, ReadSouVelRho.f90:139-212,828-890).  Every
 * gather is propagated on its own window of the model (aperture_x,
 * aperture_y).
 *
 *   Task=MOD: compute_mod (compute_function_gradient.f90:472-588): AMOD
 *     forward modelling (sinc injection, nearest-node AFWI extraction) of
 *     every gather; data= receives all traces in coordfile order.
 *   Task=MIG: compute_mig (compute_function_gradient.f90:352-470): AMOD
 *     with snapshots, then the AGRAD back-propagation of the recorded traces
 *     of traces= (nearest-node injection, AFWI imaging condition); the
 *     gathers' images and illuminations are stacked on the full grid and
 *     image= receives image / ((illum + max/10000) / rms(illum)).
 *   Task=INV needs the mute and band-pass preprocessing of the reference,
 *     which this build does not implement; it stops with an error.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "swcli.h"

typedef struct gather {
  int begi, ntr;   /* first trace (0-based) and trace count */
  float sou[3];
} gather;

static float *read_all_keys(int *nkeys_out, int *ntot_out) {
  if (!sep_exist("coordfile")) cli_fail("need coordfile");
  sep_file *f = sep_open_in("coordfile");
  if (!f) cli_fail("%s", sep_error());
  int nkeys = 0, ntot = 0;
  if (sep_hdr_int(f, "n1", &nkeys) != 1 || nkeys < 1) cli_fail("coordfile header needs n1");
  if (sep_hdr_int(f, "n2", &ntot) != 1 || ntot < 1) cli_fail("coordfile header needs n2");
  float *keys = (float *)malloc((size_t)nkeys * ntot * 4);
  if (!keys) cli_fail("out of host memory");
  if (sep_read(f, keys, (size_t)nkeys * ntot)) cli_fail("%s", sep_error());
  sep_close(f);
  *nkeys_out = nkeys;
  *ntot_out = ntot;
  return keys;
}

int main(int argc, char **argv) {
  if (sep_init(argc, argv)) cli_fail("%s", sep_error());
  if (!sep_exist("vel")) cli_fail("need velocity file");
  cli_par p;
  cli_read_params(&p);
  if (p.withRho) cli_fail("Rho not implemented in this version");
  const int mod = !strcmp(p.task, "MOD") || !strcmp(p.task, "mod");
  const int mig = !strcmp(p.task, "MIG") || !strcmp(p.task, "mig");
  if (!mod && !mig)
    cli_fail("Task=%s: only MOD and MIG are built (INV needs the mute and band-pass "
             "preprocessing, not built in swave)", p.task);
  float *wavelet = cli_read_source(&p);
  const int nt = p.g.nt;

  const char *names[6] = {"keygx", "keysx", "keygy", "keysy", "keyselev", "keygelev"};
  int idx[6];
  for (int k = 0; k < 6; ++k)
    if (sep_par_int(names[k], &idx[k]) != 1) cli_fail("need %s", names[k]);
  int nkeys = 0, ntot = 0;
  float *keys = read_all_keys(&nkeys, &ntot);
  for (int k = 0; k < 6; ++k)
    if (idx[k] < 1 || idx[k] > nkeys) cli_fail("%s=%d is outside 1..%d", names[k], idx[k], nkeys);
  float *rec = (float *)malloc((size_t)ntot * 3 * 4);
  gather *gs = (gather *)malloc((size_t)ntot * sizeof(gather));
  if (!rec || !gs) cli_fail("out of host memory");
  int ng = 0;
  for (int i = 0; i < ntot; ++i) {
    const float *k = keys + (size_t)i * nkeys;
    rec[3 * i + 0] = k[idx[5] - 1];
    rec[3 * i + 1] = k[idx[0] - 1];
    rec[3 * i + 2] = k[idx[2] - 1];
    const float sx = k[idx[1] - 1], sy = k[idx[3] - 1];
    if (ng == 0 || sx != gs[ng - 1].sou[1] || sy != gs[ng - 1].sou[2]) {
      gs[ng].begi = i;
      gs[ng].ntr = 0;
      ++ng;
    }
    gather *g = &gs[ng - 1];
    g->ntr++;
    g->sou[0] = k[idx[4] - 1];  /* the gather's last trace gives the source */
    g->sou[1] = sx;
    g->sou[2] = sy;
  }
  fprintf(stderr, "INFO: ngathers %d nkeys %d ntraces %d\n", ng, nkeys, ntot);

  float *traces = NULL;
  if (mig) {
    int ntr = 0;
    traces = cli_read_traces(nt, &ntr);
    if (ntr != ntot) cli_fail("number of read traces is different from n2 in traces");
  }
  float *vel = cli_read_model(&p, "vel");
  float cour = 0.f, sr = 0.f;
  if (sw_vel_check(&p.g, vel, &cour, &sr) != SW_OK)
    cli_fail("vel_check: Courant number %g or %g samples per minimum wavelength out of range",
             (double)cour, (double)sr);
  const char *out_tag = mod ? "data" : "image";
  if (!sep_exist(out_tag)) cli_fail("need %s file for output", out_tag);

  sw_ctx *ctx = cli_context();
  const size_t nm = (size_t)p.g.nz * p.g.nx * p.g.ny;
  float *out = (float *)calloc(mod ? (size_t)ntot * nt : nm, 4);
  float *illu = mig ? (float *)calloc(nm, 4) : NULL;
  if (!out || (mig && !illu)) cli_fail("out of host memory");
  for (int ig = 0; ig < ng; ++ig) {
    const gather *G = &gs[ig];
    const float *grec = rec + 3 * (size_t)G->begi;
    sw_window w;
    sw_genpar gw;
    cli_shot_window(&p, G->sou, G->ntr, grec, &w, &gw);
    const size_t nw = (size_t)gw.nz * gw.nx * gw.ny;
    float *vs = (float *)malloc(nw * 4);
    if (!vs) cli_fail("out of host memory");
    sw_window_extract(&p.g, &w, vel, vs);
    sw_prop_desc fd;
    memset(&fd, 0, sizeof(fd));
    fd.g = gw;
    fd.tmin = 1;
    fd.tmax = nt;
    fd.tstep = 1;
    fd.fd_scheme = SW_FD_FORWARD;
    fd.injection = SW_INJ_SINC;
    sw_prop_io a;
    memset(&a, 0, sizeof(a));
    a.vel = vs;
    a.nsou = 1;
    a.sou_coord = G->sou;
    a.sou_trace = wavelet;
    if (mod) {
      /* AMOD_to_memory (to_disk_to_memory_AMOD.f90:27-82). */
      fd.extraction = SW_EXT_SIMPLE_AFWI;
      a.nrec = G->ntr;
      a.rec_coord = grec;
      a.rec_trace = out + (size_t)G->begi * nt;
      cli_check(ctx, sw_propagate(ctx, &fd, &a), "AMOD propagation");
    } else {
      const int ntsnap = nt / gw.snapi;
      float *wave = (float *)malloc(nw * (size_t)(ntsnap > 0 ? ntsnap : 1) * 4);
      float *ims = (float *)calloc(nw, 4), *ils = (float *)calloc(nw, 4);
      if (!wave || !ims || !ils) cli_fail("out of host memory");
      fd.extract_wave = 1;
      a.wave = wave;
      cli_check(ctx, sw_propagate(ctx, &fd, &a), "AMOD propagation");
      /* AGRAD_to_memory (to_disk_to_memory_AGRAD.f90:27-79). */
      sw_prop_desc bd;
      memset(&bd, 0, sizeof(bd));
      bd.g = gw;
      bd.tmin = nt;
      bd.tmax = 1;
      bd.tstep = -1;
      bd.fd_scheme = SW_FD_FORWARD;
      bd.injection = SW_INJ_SIMPLE;
      bd.imaging = SW_IMG_AFWI;
      sw_prop_io b;
      memset(&b, 0, sizeof(b));
      b.vel = vs;
      b.nsou = G->ntr;
      b.sou_coord = grec;
      b.sou_trace = traces + (size_t)G->begi * nt;
      b.wave = wave;
      b.image = ims;
      b.illum = ils;
      cli_check(ctx, sw_propagate(ctx, &bd, &b), "AGRAD propagation");
      sw_window_scatter_add(&p.g, &w, ims, out);
      sw_window_scatter_add(&p.g, &w, ils, illu);
      free(wave);
      free(ims);
      free(ils);
    }
    free(vs);
    if ((ig + 1) % 10 == 0) fprintf(stderr, "INFO: %d of %d gathers done\n", ig + 1, ng);
  }

  sep_file *f = sep_open_out(out_tag);
  if (!f) cli_fail("%s", sep_error());
  if (mod) {
    if (sep_write(f, out, (size_t)ntot * nt)) cli_fail("%s", sep_error());
    sep_put_int(f, "n1", nt);
    sep_put_int(f, "n2", ntot);
    sep_put_float(f, "d1", p.g.dt);
    sep_put_float(f, "d2", 1.f);
    sep_put_float(f, "o1", 0.f);
    sep_put_float(f, "o2", 0.f);
  } else {
    /* illu = (illu + maxval(illu)/10000) / sqrt(sum(dprod(illu,illu))/size(illu));
     * imag = imag/illu (compute_function_gradient.f90:452-453). */
    float mx = illu[0];
    double ss = 0.0;
    for (size_t q = 0; q < nm; ++q) {
      mx = illu[q] > mx ? illu[q] : mx;
      ss += (double)illu[q] * (double)illu[q];
    }
    const double r = sqrt(ss / (double)nm);
    for (size_t q = 0; q < nm; ++q) {
      const float v = (float)((double)(illu[q] + mx / 10000.f) / r);
      out[q] = out[q] / v;
    }
    if (sep_write(f, out, nm)) cli_fail("%s", sep_error());
    sep_put_int(f, "n1", p.g.nz);
    sep_put_int(f, "n2", p.g.nx);
    sep_put_int(f, "n3", p.g.ny);
  }
  if (sep_close(f)) cli_fail("%s", sep_error());
  sw_ctx_destroy(ctx);
  free(out);
  free(illu);
  free(vel);
  free(traces);
  free(rec);
  free(gs);
  free(keys);
  free(wavelet);
  sep_finish();
  return 0;
}
