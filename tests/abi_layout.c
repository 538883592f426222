/* Prints the layout of every struct of include/swave.h: one line per struct
 * ("struct <name> <sizeof>") followed by one line per field in declaration
 * order ("field <name> <offsetof> <sizeof>").  Built and run by
 * tests/test_abi_layout.py, which compares it with the ctypes mirror
 * (seismic_gb300/__init__.py) and the Fortran bind(C) types
 * (include/swave_iface.f90). */
#include <stddef.h>
#include <stdio.h>

#include "swave.h"

#define S(T) printf("struct %s %zu\n", #T, sizeof(T))
#define F(T, f) printf("field %s %zu %zu\n", #f, offsetof(T, f), sizeof(((T *)0)->f))

int main(void) {
  S(sw_genpar);
  F(sw_genpar, twoD); F(sw_genpar, nz); F(sw_genpar, nx); F(sw_genpar, ny);
  F(sw_genpar, dz); F(sw_genpar, dx); F(sw_genpar, dy);
  F(sw_genpar, oz); F(sw_genpar, ox); F(sw_genpar, oy); F(sw_genpar, dt);
  F(sw_genpar, nt); F(sw_genpar, ntaper); F(sw_genpar, lsinc); F(sw_genpar, snapi);
  F(sw_genpar, surf_type); F(sw_genpar, shot_type); F(sw_genpar, rec_type); F(sw_genpar, fmax);

  S(sw_prop_desc);
  F(sw_prop_desc, g); F(sw_prop_desc, tmin); F(sw_prop_desc, tmax); F(sw_prop_desc, tstep);
  F(sw_prop_desc, fd_scheme); F(sw_prop_desc, injection); F(sw_prop_desc, extraction);
  F(sw_prop_desc, extract_wave); F(sw_prop_desc, imaging);

  S(sw_prop_io);
  F(sw_prop_io, vel); F(sw_prop_io, nsou); F(sw_prop_io, sou_coord); F(sw_prop_io, sou_trace);
  F(sw_prop_io, nrec); F(sw_prop_io, rec_coord); F(sw_prop_io, rec_trace); F(sw_prop_io, wave);
  F(sw_prop_io, image); F(sw_prop_io, illum); F(sw_prop_io, ref); F(sw_prop_io, final_u2);
  F(sw_prop_io, rho); F(sw_prop_io, image2);

  S(sw_shot);
  F(sw_shot, sou_coord); F(sw_shot, nrec); F(sw_shot, rec_coord); F(sw_shot, data);
  F(sw_shot, nt);

  S(sw_window);
  F(sw_window, oxw); F(sw_window, oyw); F(sw_window, endx); F(sw_window, endy);
  F(sw_window, nxw); F(sw_window, nyw);

  S(sw_fwi_shot);
  F(sw_fwi_shot, sou_coord); F(sw_fwi_shot, nrec); F(sw_fwi_shot, rec_coord);
  F(sw_fwi_shot, dobs); F(sw_fwi_shot, mute); F(sw_fwi_shot, resid);

  S(sw_fwi_desc);
  F(sw_fwi_desc, g); F(sw_fwi_desc, aperture_x); F(sw_fwi_desc, aperture_y);
  F(sw_fwi_desc, illu_pow); F(sw_fwi_desc, smooth_rect1); F(sw_fwi_desc, smooth_rect2);
  F(sw_fwi_desc, smooth_rect3); F(sw_fwi_desc, smooth_doz); F(sw_fwi_desc, smooth_dox);
  F(sw_fwi_desc, smooth_doy); F(sw_fwi_desc, checkpoint_snaps); F(sw_fwi_desc, dat_nrm_type);
  F(sw_fwi_desc, dat_thresh); F(sw_fwi_desc, revolve_slots);

  S(sw_reg_desc);
  F(sw_reg_desc, nz); F(sw_reg_desc, nx); F(sw_reg_desc, ny); F(sw_reg_desc, wantreg);
  F(sw_reg_desc, wantlog); F(sw_reg_desc, derivdx); F(sw_reg_desc, derivdy);
  F(sw_reg_desc, derivdz); F(sw_reg_desc, log_z_plus); F(sw_reg_desc, ntaperz);
  F(sw_reg_desc, ntaperx); F(sw_reg_desc, ntapery); F(sw_reg_desc, mod_nrm_type);
  F(sw_reg_desc, hin_nrm_type); F(sw_reg_desc, compute_eps); F(sw_reg_desc, compute_eps_log);
  F(sw_reg_desc, ratio); F(sw_reg_desc, ratio_log); F(sw_reg_desc, zweight);

  S(sw_reg_state);
  F(sw_reg_state, eps); F(sw_reg_state, eps_log); F(sw_reg_state, mod_thresh);
  F(sw_reg_state, hin_thresh);

  S(sw_lbfgs_oc_state);
  F(sw_lbfgs_oc_state, gtol); F(sw_lbfgs_oc_state, one); F(sw_lbfgs_oc_state, zero);
  F(sw_lbfgs_oc_state, gnorm); F(sw_lbfgs_oc_state, stp1); F(sw_lbfgs_oc_state, ftol);
  F(sw_lbfgs_oc_state, stpmin); F(sw_lbfgs_oc_state, stpmax); F(sw_lbfgs_oc_state, stp);
  F(sw_lbfgs_oc_state, ys); F(sw_lbfgs_oc_state, yy); F(sw_lbfgs_oc_state, sq);
  F(sw_lbfgs_oc_state, yr); F(sw_lbfgs_oc_state, beta); F(sw_lbfgs_oc_state, xnorm);
  F(sw_lbfgs_oc_state, mp); F(sw_lbfgs_oc_state, lp); F(sw_lbfgs_oc_state, iter);
  F(sw_lbfgs_oc_state, nfun); F(sw_lbfgs_oc_state, point); F(sw_lbfgs_oc_state, ispt);
  F(sw_lbfgs_oc_state, iypt); F(sw_lbfgs_oc_state, maxfev); F(sw_lbfgs_oc_state, info);
  F(sw_lbfgs_oc_state, bound); F(sw_lbfgs_oc_state, npt); F(sw_lbfgs_oc_state, cp);
  F(sw_lbfgs_oc_state, i); F(sw_lbfgs_oc_state, nfev); F(sw_lbfgs_oc_state, inmc);
  F(sw_lbfgs_oc_state, iycn); F(sw_lbfgs_oc_state, iscn); F(sw_lbfgs_oc_state, finish);
  F(sw_lbfgs_oc_state, infoc); F(sw_lbfgs_oc_state, j); F(sw_lbfgs_oc_state, brackt);
  F(sw_lbfgs_oc_state, stage1); F(sw_lbfgs_oc_state, dg); F(sw_lbfgs_oc_state, dgm);
  F(sw_lbfgs_oc_state, dginit); F(sw_lbfgs_oc_state, dgtest); F(sw_lbfgs_oc_state, dgx);
  F(sw_lbfgs_oc_state, dgxm); F(sw_lbfgs_oc_state, dgy); F(sw_lbfgs_oc_state, dgym);
  F(sw_lbfgs_oc_state, finit); F(sw_lbfgs_oc_state, ftest1); F(sw_lbfgs_oc_state, fm);
  F(sw_lbfgs_oc_state, fx); F(sw_lbfgs_oc_state, fxm); F(sw_lbfgs_oc_state, fy);
  F(sw_lbfgs_oc_state, fym); F(sw_lbfgs_oc_state, stx); F(sw_lbfgs_oc_state, sty);
  F(sw_lbfgs_oc_state, stmin); F(sw_lbfgs_oc_state, stmax); F(sw_lbfgs_oc_state, width);
  F(sw_lbfgs_oc_state, width1);

  S(sw_lbfgs_oc_desc);
  F(sw_lbfgs_oc_desc, n); F(sw_lbfgs_oc_desc, m); F(sw_lbfgs_oc_desc, nparam);
  F(sw_lbfgs_oc_desc, xmin); F(sw_lbfgs_oc_desc, xmax); F(sw_lbfgs_oc_desc, lbfgs_type);
  F(sw_lbfgs_oc_desc, bound_type); F(sw_lbfgs_oc_desc, stp1_opt); F(sw_lbfgs_oc_desc, step_init);
  F(sw_lbfgs_oc_desc, eps); F(sw_lbfgs_oc_desc, xtol);

  S(sw_tuning);
  F(sw_tuning, step_kernel); F(sw_tuning, tile_z); F(sw_tuning, tile_x); F(sw_tuning, tile_y);
  F(sw_tuning, graph_chunk); F(sw_tuning, use_graph);

  S(sw_stats);
  F(sw_stats, launches_total); F(sw_stats, launches_step); F(sw_stats, points_updated);
  F(sw_stats, step_kernel_ms); F(sw_stats, step_kernel_timed); F(sw_stats, step_bytes);
  F(sw_stats, steps_forward); F(sw_stats, steps_backward); F(sw_stats, ckpt_advances);
  F(sw_stats, cnn_conv_ms); F(sw_stats, cnn_conv_timed); F(sw_stats, cnn_conv_bytes);
  F(sw_stats, cnn_conv_flops);
  return 0;
}
