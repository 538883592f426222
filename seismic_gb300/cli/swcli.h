/* swcli.h - the reading steps shared by the swave command-line programs,
 * on top of sep.h and the libswave C ABI. */
#ifndef SWAVE_CLI_H
#define SWAVE_CLI_H

#include "../../include/swave.h"
#include "sep.h"

typedef struct cli_par {
  sw_genpar g; /* full model grid; dt and nt from the wavelet */
  float aperture_x, aperture_y;
  int withRho, LSRTM, CHEAPLSRTM, Born, verbose, nthreads, WriteFwdWvfld;
  float max_memory;
  char task[32];
} cli_par;

/* Prints "ERROR: ..." to standard error and exits with status 1 (erexit). */
void cli_fail(const char *fmt, ...);

/* read_3D_params (libs/libwave/ReadParam.f90:15-84): fmax 30, ntaper 20,
 * snapi 4, lsinc 7, num_threads 4, maxsize 16, rec/shot/surf_type 0, twoD,
 * withRho, LSRTM, Born false, verb true, Task MOD.  Programs without a
 * variable-density path reject withRho themselves. */
void cli_read_params(cli_par *p);

/* readsou (ReadSouVelRho.f90:298-344): the wavelet from the "in" dataset
 * (n1 = nt, d1 = dt, o1 = t0); with Born or LSRTM it is replaced by its
 * centred second difference / dt^2, with withRho it is then moved half a
 * sample (sw_rho_wavelet).  Returns the nt samples (malloc). */
float *cli_read_source(cli_par *p);

/* readtraces (ReadSouVelRho.f90:59-88): n2 traces of n1 = nt samples from
 * the "traces" dataset.  Returns them (malloc, ntr*nt), sets *ntr and, when
 * ot is not NULL, the first sample's time (o1). */
float *cli_read_traces(int nt, int *ntr, float *ot);

/* readcoords (ReadSouVelRho.f90:90-137): coordfile rows of n1 keys, one per
 * trace; keygelev/keygx/keygy give the receiver (z, x, y), the last row's
 * keyselev/keysx/keysy the source.  Returns 3*ntr receiver coordinates
 * (malloc) and fills sou[3]. */
float *cli_read_coords(int ntr, float sou[3]);

/* The model dataset `tag` (read_window_vel, ExtractPadModel.f90:87-131):
 * n1/o1/d1, n2/o2/d2 and, in 3D, n3/o3/d3 into p->g (the first call) or
 * checked against p->g (later calls: dim_consistency_check).  Returns the
 * nz*nx*ny samples (malloc). */
float *cli_read_model(cli_par *p, const char *tag);

/* The shot's window (extract_coord_source_receiver_patch) with the check of
 * read_window_vel (ExtractPadModel.f90:151-174): the patch may not lie
 * outside the model on every side.  *gw receives the window's genpar. */
void cli_shot_window(const cli_par *p, const float sou[3], int ntr, const float *rec,
                     sw_window *w, sw_genpar *gw);

/* Writes nz*nx*ny image then illumination with 3DRTM's header
 * (progs/rtm/3DRTM.f90:131-146). */
void cli_write_image(const cli_par *p, const char *tag, const float *image, const float *illum);

/* Writes ntr traces with the data header of Acoustic_modeling_sep and
 * 3DBORNMOD (n1 = nt, n2 = ntr, d1 = dt, d2 = 1, o1 = o2 = 0). */
void cli_write_traces(const cli_par *p, const char *tag, int ntr, const float *data);

/* A context on device 0 (fails loudly without a CUDA device). */
sw_ctx *cli_context(void);
void cli_check(sw_ctx *ctx, int status, const char *what);

#endif
