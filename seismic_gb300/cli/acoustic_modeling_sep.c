/* Acoustic_modeling_sep.x - forward modelling of one shot
 * (progs/modeling/Acoustic_modeling_sep.f90): the wavelet from stdin=
 * (or standard input), receivers from traces= (record length and count) and
 * coordfile= (keygx, keysx, ...), the model from vel=; the shot's window of
 * the model (source/receiver patch widened by aperture_x/aperture_y) is
 * propagated on the GPU with sinc injection and sinc extraction; the traces
 * go to data=.
 *
 *   Acoustic_modeling_sep.x stdin=wavelet.H vel=vel.H traces=t.H \
 *       coordfile=keys.H keygx=.. keysx=.. keygy=.. keysy=.. keyselev=.. \
 *       keygelev=.. aperture_x=.. aperture_y=.. twoD=1 data=out.H
 */
#include <stdlib.h>

#include "swcli.h"

int main(int argc, char **argv) {
  if (sep_init(argc, argv)) cli_fail("%s", sep_error());
  cli_par p;
  cli_read_params(&p);
  float *wavelet = cli_read_source(&p);
  int ntr = 0;
  float *traces = cli_read_traces(p.g.nt, &ntr);
  float sou[3];
  float *rec = cli_read_coords(ntr, sou);
  float *vel = cli_read_model(&p, "vel");
  if (!sep_exist("data")) cli_fail("need data file for output");
  sw_window w;
  sw_genpar gw;
  cli_shot_window(&p, sou, ntr, rec, &w, &gw);
  float cour = 0.f, sr = 0.f;
  if (sw_vel_check(&p.g, vel, &cour, &sr) != SW_OK)
    cli_fail("vel_check: Courant number %g or %g samples per minimum wavelength out of range",
             (double)cour, (double)sr);
  float *vsmall = (float *)malloc((size_t)gw.nz * gw.nx * gw.ny * 4);
  if (!vsmall || sw_window_extract(&p.g, &w, vel, vsmall) != SW_OK) cli_fail("window extract");
  sw_ctx *ctx = cli_context();
  cli_check(ctx, sw_modeling(ctx, &gw, vsmall, sou, wavelet, ntr, rec, traces, NULL),
            "sw_modeling");
  cli_write_traces(&p, "data", ntr, traces);
  sw_ctx_destroy(ctx);
  free(vsmall);
  free(vel);
  free(rec);
  free(traces);
  free(wavelet);
  sep_finish();
  return 0;
}
