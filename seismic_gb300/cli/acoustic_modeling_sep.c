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
 *
 * withRho=1 with rho=density.H (same grid as vel=) runs the
 * variable-density operator (FD_{2D,3D}_derivatives_acoustic_forward_grid)
 * with the wavelet moved half a sample.
 */
#include <stdlib.h>
#include <string.h>

#include "swcli.h"

int main(int argc, char **argv) {
  if (sep_init(argc, argv)) cli_fail("%s", sep_error());
  cli_par p;
  cli_read_params(&p);
  float *wavelet = cli_read_source(&p);
  int ntr = 0;
  float *traces = cli_read_traces(p.g.nt, &ntr, NULL);
  float sou[3];
  float *rec = cli_read_coords(ntr, sou);
  float *vel = cli_read_model(&p, "vel");
  float *rho = p.withRho ? cli_read_model(&p, "rho") : NULL;
  if (!sep_exist("data")) cli_fail("need data file for output");
  sw_window w;
  sw_genpar gw;
  cli_shot_window(&p, sou, ntr, rec, &w, &gw);
  float cour = 0.f, sr = 0.f;
  if (sw_vel_check(&p.g, vel, &cour, &sr) != SW_OK)
    cli_fail("vel_check: Courant number %g or %g samples per minimum wavelength out of range",
             (double)cour, (double)sr);
  const size_t nw = (size_t)gw.nz * gw.nx * gw.ny;
  float *vsmall = (float *)malloc(nw * 4);
  if (!vsmall || sw_window_extract(&p.g, &w, vel, vsmall) != SW_OK) cli_fail("window extract");
  float *rsmall = NULL;
  if (rho) {
    rsmall = (float *)malloc(nw * 4);
    if (!rsmall || sw_window_extract(&p.g, &w, rho, rsmall) != SW_OK) cli_fail("window extract");
  }
  sw_ctx *ctx = cli_context();
  if (!rho) {
    cli_check(ctx, sw_modeling(ctx, &gw, vsmall, sou, wavelet, ntr, rec, traces, NULL),
              "sw_modeling");
  } else {
    /* propagator_acoustic with FD_acoustic_rho_init_coefs and
     * FD_*_derivatives_acoustic_forward_grid (Acoustic_modeling_sep.f90:
     * 93-104, 118-129). */
    sw_prop_desc d;
    memset(&d, 0, sizeof(d));
    d.g = gw;
    d.tmin = 1;
    d.tmax = gw.nt;
    d.tstep = 1;
    d.fd_scheme = SW_FD_FORWARD;
    d.injection = SW_INJ_SINC;
    d.extraction = SW_EXT_SINC;
    sw_prop_io io;
    memset(&io, 0, sizeof(io));
    io.vel = vsmall;
    io.rho = rsmall;
    io.nsou = 1;
    io.sou_coord = sou;
    io.sou_trace = wavelet;
    io.nrec = ntr;
    io.rec_coord = rec;
    memset(traces, 0, (size_t)ntr * gw.nt * 4);
    io.rec_trace = traces;
    cli_check(ctx, sw_propagate(ctx, &d, &io), "sw_propagate (withRho)");
  }
  cli_write_traces(&p, "data", ntr, traces);
  sw_ctx_destroy(ctx);
  free(vsmall);
  free(rsmall);
  free(rho);
  free(vel);
  free(rec);
  free(traces);
  free(wavelet);
  sep_finish();
  return 0;
}
