/* 3DRTM.x - RTM (or, with LSRTM=1, the LSRTM adjoint) of one shot
 * (progs/rtm/3DRTM.f90): the wavelet from stdin= (second-differenced when
 * Born=1 or LSRTM=1), the recorded traces from traces=, their keys from
 * coordfile=, the model from vel=.  The shot's window is migrated on the
 * GPU and its image and illumination are added into the full grid
 * (mod_copy_image_to_disk); image= receives the image, then the
 * illumination (n3 = 2 in 2D, n4 = 2 in 3D).  Snapshots stay in device
 * memory: maxsize= and the wave_fwd disk path of the reference are not
 * used. */
#include <stdlib.h>
#include <string.h>

#include "swcli.h"

int main(int argc, char **argv) {
  if (sep_init(argc, argv)) cli_fail("%s", sep_error());
  if (!sep_exist("vel")) cli_fail("need vel file");
  if (sep_exist("vel2")) cli_fail("vel2= (a second velocity) is not built in swave");
  cli_par p;
  cli_read_params(&p);
  float *wavelet = cli_read_source(&p);
  int ntr = 0;
  float *traces = cli_read_traces(p.g.nt, &ntr);
  float sou[3];
  float *rec = cli_read_coords(ntr, sou);
  float *vel = cli_read_model(&p, "vel");
  if (!sep_exist("image")) cli_fail("need image file for output");
  sw_window w;
  sw_genpar gw;
  cli_shot_window(&p, sou, ntr, rec, &w, &gw);
  float cour = 0.f, sr = 0.f;
  if (sw_vel_check(&p.g, vel, &cour, &sr) != SW_OK)
    cli_fail("vel_check: Courant number %g or %g samples per minimum wavelength out of range",
             (double)cour, (double)sr);
  const size_t nw = (size_t)gw.nz * gw.nx * gw.ny;
  const size_t nm = (size_t)p.g.nz * p.g.nx * p.g.ny;
  float *vsmall = (float *)malloc(nw * 4);
  float *ims = (float *)malloc(nw * 4), *ils = (float *)malloc(nw * 4);
  float *im = (float *)calloc(nm, 4), *il = (float *)calloc(nm, 4);
  if (!vsmall || !ims || !ils || !im || !il) cli_fail("out of host memory");
  if (sw_window_extract(&p.g, &w, vel, vsmall) != SW_OK) cli_fail("window extract");
  sw_ctx *ctx = cli_context();
  if (p.LSRTM)
    cli_check(ctx, sw_lsrtm(ctx, &gw, vsmall, sou, wavelet, ntr, rec, traces, ims, ils),
              "sw_lsrtm");
  else
    cli_check(ctx, sw_rtm(ctx, &gw, vsmall, sou, wavelet, ntr, rec, traces, ims, ils), "sw_rtm");
  sw_window_scatter_add(&p.g, &w, ims, im);
  sw_window_scatter_add(&p.g, &w, ils, il);
  cli_write_image(&p, "image", im, il);
  sw_ctx_destroy(ctx);
  free(vsmall);
  free(ims);
  free(ils);
  free(im);
  free(il);
  free(vel);
  free(rec);
  free(traces);
  free(wavelet);
  sep_finish();
  return 0;
}
