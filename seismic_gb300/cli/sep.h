/* sep.h - SEP dataset and parameter I/O for the swave command-line programs.
 *
 * A SEP dataset is a text header ("history") of name=value pairs plus a
 * binary file named by the header's in= value.  The header lines of every
 * program that touched the dataset are kept; a later definition of a name
 * overrides an earlier one.  Samples are 4-byte floats, big-endian when
 * data_format="xdr_float" (the default when the header names none) and
 * little-endian when data_format="native_float".  A header whose in= is
 * "stdin" (or absent) carries its samples after a form-feed + EOT (0x0c 0x04)
 * marker in the same file.
 *
 * Parameters come from the command line (name=value words; par=file reads
 * more name=value pairs from a file); a later definition overrides an
 * earlier one.  A dataset named by a tag is given on the command line as
 * tag=path; the "in" dataset is stdin=path or, failing that, standard input.
 * These follow the calls the reference programs make (from_param, from_aux,
 * from_history, sreed, srite, to_history, exist_file in progs/rtm/3DRTM.f90,
 * progs/modeling/Acoustic_modeling_sep.f90, libs/libwave/ReadSouVelRho.f90).
 */
#ifndef SWAVE_SEP_H
#define SWAVE_SEP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Records the program name and the command line's parameters (expanding
 * par= files).  Returns 0, or -1 when a par= file cannot be read. */
int sep_init(int argc, char **argv);
void sep_finish(void);

/* Parameter lookup (from_param).  Each returns 1 when the name is present
 * and parses, 0 when absent (the value is left untouched) and -1 when the
 * value does not parse. */
int sep_par_str(const char *name, char *out, size_t n);
int sep_par_int(const char *name, int *v);
int sep_par_float(const char *name, float *v);
/* y/yes/t/true/.true./1 and n/no/f/false/.false./0, any case. */
int sep_par_bool(const char *name, int *v);

/* exist_file: the tag names a dataset on the command line ("in": stdin=
 * given, or standard input is not a terminal). */
int sep_exist(const char *tag);

typedef struct sep_file sep_file;

/* Opens the dataset of `tag` for sequential reading.  NULL on failure
 * (sep_error() says why). */
sep_file *sep_open_in(const char *tag);
/* Opens the dataset of `tag` (tag=path on the command line) for writing:
 * the header goes to path, the samples to the datapath= parameter (or the
 * DATAPATH environment variable) + the header's base name + "@", else to
 * path + "@". */
sep_file *sep_open_out(const char *tag);

/* Header values (from_aux / from_history / auxpar).  Same return
 * convention as the parameter lookups. */
int sep_hdr_str(const sep_file *f, const char *name, char *out, size_t n);
int sep_hdr_int(const sep_file *f, const char *name, int *v);
int sep_hdr_float(const sep_file *f, const char *name, float *v);

/* Sequential samples (sreed / srite).  Return 0 or -1. */
int sep_read(sep_file *f, float *buf, size_t n);
int sep_write(sep_file *f, const float *buf, size_t n);

/* Output header values (to_history), written when the file is closed. */
int sep_put_int(sep_file *f, const char *name, int v);
int sep_put_float(sep_file *f, const char *name, float v);
int sep_put_str(sep_file *f, const char *name, const char *v);

/* Closes the dataset; an output dataset's header is written here.
 * Returns 0 or -1. */
int sep_close(sep_file *f);

const char *sep_error(void);

#ifdef __cplusplus
}
#endif

#endif
