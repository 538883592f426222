/* 3DBORNMOD.x - Born modelling of one shot (progs/modeling/3DBORNMOD.f90):
 * the wavelet from stdin= (second-differenced: Born is always on), the
 * record length and receiver count from traces=, their keys from
 * coordfile=, the background model from vel= and the reflectivity from
 * ref= (same grid).  The shot's windows of both are propagated on the GPU
 * (BORN_to_memory); data= receives the scattered traces. */
#include <stdlib.h>

#include "swcli.h"

int main(int argc, char **argv) {
  if (sep_init(argc, argv)) cli_fail("%s", sep_error());
  if (!sep_exist("vel")) cli_fail("need velocity file");
  if (!sep_exist("ref")) cli_fail("need reflectivity file");
  if (!sep_exist("data")) cli_fail("need dat file for output");
  cli_par p;
  cli_read_params(&p);
  if (p.withRho) cli_fail("withRho=1: Born modelling has no variable-density path in swave");
  p.Born = 1;
  float *wavelet = cli_read_source(&p);
  int ntr = 0;
  float *traces = cli_read_traces(p.g.nt, &ntr, NULL);
  float sou[3];
  float *rec = cli_read_coords(ntr, sou);
  float *vel = cli_read_model(&p, "vel");
  float *ref = cli_read_model(&p, "ref");
  sw_window w;
  sw_genpar gw;
  cli_shot_window(&p, sou, ntr, rec, &w, &gw);
  float cour = 0.f, sr = 0.f;
  if (sw_vel_check(&p.g, vel, &cour, &sr) != SW_OK)
    cli_fail("vel_check: Courant number %g or %g samples per minimum wavelength out of range",
             (double)cour, (double)sr);
  const size_t nw = (size_t)gw.nz * gw.nx * gw.ny;
  float *vsmall = (float *)malloc(nw * 4), *rsmall = (float *)malloc(nw * 4);
  if (!vsmall || !rsmall) cli_fail("out of host memory");
  if (sw_window_extract(&p.g, &w, vel, vsmall) != SW_OK ||
      sw_window_extract(&p.g, &w, ref, rsmall) != SW_OK)
    cli_fail("window extract");
  sw_ctx *ctx = cli_context();
  cli_check(ctx, sw_born(ctx, &gw, vsmall, rsmall, sou, wavelet, ntr, rec, traces), "sw_born");
  cli_write_traces(&p, "data", ntr, traces);
  sw_ctx_destroy(ctx);
  free(vsmall);
  free(rsmall);
  free(ref);
  free(vel);
  free(rec);
  free(traces);
  free(wavelet);
  sep_finish();
  return 0;
}
