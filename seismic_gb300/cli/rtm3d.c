/* 3DRTM.x - RTM (or, with LSRTM=1, the LSRTM adjoint) of one shot
 * (progs/rtm/3DRTM.f90): the wavelet from stdin= (second-differenced when
 * Born=1 or LSRTM=1), the recorded traces from traces=, their keys from
 * coordfile=, the model from vel=.  The shot's window is migrated on the
 * GPU and its image and illumination are added into the full grid
 * (mod_copy_image_to_disk); image= receives the image, then the
 * illumination (n3 = 2 in 2D, n4 = 2 in 3D).  Snapshots stay in device
 * memory: maxsize= and the wave_fwd disk path of the reference are not
 * used.  withRho=1 with rho= runs RTM_to_memory's variable-density branch:
 * the forward-grid density operator in both passes
 * (to_disk_to_memory_RTM.f90:388-398,455-465).  LSRTM=1 CHEAPLSRTM=1 runs
 * CHEAP_LSRTM_to_memory (to_disk_to_memory_RTM.f90:581-668): the LSRTM
 * backward pass on the forward-grid stencil instead of the adjoint one.
 * vel2= replaces the velocity of the backward pass and of its imaging
 * condition (mod%vel=mod%vel2, to_disk_to_memory_RTM.f90:438-439,550-551,
 * 637-638); the passes then run as two sw_propagate calls with the
 * procedures sw_rtm / sw_lsrtm use. */
#include <stdlib.h>
#include <string.h>

#include "swcli.h"

int main(int argc, char **argv) {
  if (sep_init(argc, argv)) cli_fail("%s", sep_error());
  if (!sep_exist("vel")) cli_fail("need vel file");
  cli_par p;
  cli_read_params(&p);
  float *wavelet = cli_read_source(&p);
  int ntr = 0;
  float *traces = cli_read_traces(p.g.nt, &ntr, NULL);
  float sou[3];
  float *rec = cli_read_coords(ntr, sou);
  if (p.withRho && p.LSRTM) cli_fail("withRho=1 with LSRTM=1 is not built in swave");
  float *vel = cli_read_model(&p, "vel");
  float *rho = p.withRho ? cli_read_model(&p, "rho") : NULL;
  float *vel2 = sep_exist("vel2") ? cli_read_model(&p, "vel2") : NULL;
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
  if (rho || p.CHEAPLSRTM || vel2) {
    float *rs = NULL, *vsmall2 = NULL;
    const int ntsnap = gw.nt / gw.snapi;
    float *wave = (float *)malloc(nw * (size_t)(ntsnap > 0 ? ntsnap : 1) * 4);
    if (!wave) cli_fail("out of host memory");
    if (rho) {
      rs = (float *)malloc(nw * 4);
      if (!rs || sw_window_extract(&p.g, &w, rho, rs) != SW_OK) cli_fail("window extract");
    }
    if (vel2) {
      vsmall2 = (float *)malloc(nw * 4);
      if (!vsmall2 || sw_window_extract(&p.g, &w, vel2, vsmall2) != SW_OK)
        cli_fail("window extract");
    }
    sw_prop_desc d;
    memset(&d, 0, sizeof(d));
    d.g = gw;
    d.tmin = 1;
    d.tmax = gw.nt;
    d.tstep = 1;
    d.fd_scheme = SW_FD_FORWARD;
    d.injection = SW_INJ_SINC;
    d.extract_wave = 1;
    sw_prop_io io;
    memset(&io, 0, sizeof(io));
    io.vel = vsmall;
    io.rho = rs;
    io.nsou = 1;
    io.sou_coord = sou;
    io.sou_trace = wavelet;
    io.wave = wave;
    cli_check(ctx, sw_propagate(ctx, &d, &io), "forward propagation");
    d.tmin = gw.nt;
    d.tmax = 1;
    d.tstep = -1;
    d.extract_wave = 0;
    d.imaging = p.LSRTM ? SW_IMG_LSRTM : SW_IMG_RTM;
    d.injection = p.LSRTM ? SW_INJ_LSRTM_SINC : SW_INJ_SINC;
    /* The backward stencil of RTM_to_memory / LSRTM_to_memory: the adjoint
     * grid (RTM in 3D: the forward grid); the forward grid with rho or
     * CHEAP_LSRTM. */
    if (rho || p.CHEAPLSRTM) d.fd_scheme = SW_FD_FORWARD;
    else if (p.LSRTM) d.fd_scheme = SW_FD_ADJOINT;
    else d.fd_scheme = gw.twoD ? SW_FD_ADJOINT : SW_FD_FORWARD;
    if (vsmall2) io.vel = vsmall2;
    memset(ims, 0, nw * 4);
    memset(ils, 0, nw * 4);
    io.nsou = ntr;
    io.sou_coord = rec;
    io.sou_trace = traces;
    io.image = ims;
    io.illum = ils;
    cli_check(ctx, sw_propagate(ctx, &d, &io), "backward propagation");
    free(wave);
    free(rs);
    free(vsmall2);
  } else if (p.LSRTM)
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
  free(rho);
  free(vel2);
  free(vel);
  free(rec);
  free(traces);
  free(wavelet);
  sep_finish();
  return 0;
}
