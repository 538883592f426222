/* sep.c - SEP dataset and parameter I/O (see sep.h). */
#define _POSIX_C_SOURCE 200809L
#include "sep.h"

#include <ctype.h>
#include <errno.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ---- name=value lists ------------------------------------------------- */
typedef struct {
  char **k, **v;
  size_t n, cap;
} kvlist;

static void kv_add(kvlist *l, const char *k, size_t kn, const char *v, size_t vn) {
  if (l->n == l->cap) {
    l->cap = l->cap ? 2 * l->cap : 32;
    l->k = (char **)realloc(l->k, l->cap * sizeof(char *));
    l->v = (char **)realloc(l->v, l->cap * sizeof(char *));
  }
  l->k[l->n] = strndup(k, kn);
  l->v[l->n] = strndup(v, vn);
  l->n++;
}

static void kv_free(kvlist *l) {
  for (size_t i = 0; i < l->n; ++i) {
    free(l->k[i]);
    free(l->v[i]);
  }
  free(l->k);
  free(l->v);
  memset(l, 0, sizeof(*l));
}

/* The last definition wins. */
static const char *kv_get(const kvlist *l, const char *k) {
  for (size_t i = l->n; i-- > 0;)
    if (strcmp(l->k[i], k) == 0) return l->v[i];
  return NULL;
}

static int name_char(int c) { return isalnum(c) || c == '_' || c == '.' || c == '-'; }

/* Adds every name=value word of `text` (values optionally quoted with " or
 * '; a quoted value may hold blanks). */
static void parse_pairs(const char *text, size_t len, kvlist *l) {
  size_t i = 0;
  while (i < len) {
    while (i < len && isspace((unsigned char)text[i])) ++i;
    size_t w = i;
    while (i < len && name_char((unsigned char)text[i])) ++i;
    if (i < len && i > w && text[i] == '=') {
      const size_t kn = i - w;
      ++i;
      if (i < len && (text[i] == '"' || text[i] == '\'')) {
        const char q = text[i++];
        const size_t vs = i;
        while (i < len && text[i] != q && text[i] != '\n') ++i;
        kv_add(l, text + w, kn, text + vs, i - vs);
        if (i < len && text[i] == q) ++i;
      } else {
        const size_t vs = i;
        while (i < len && !isspace((unsigned char)text[i])) ++i;
        kv_add(l, text + w, kn, text + vs, i - vs);
      }
    }
    while (i < len && !isspace((unsigned char)text[i])) ++i; /* rest of the word */
  }
}

/* ---- errors ----------------------------------------------------------- */
static char g_err[1024];

static void set_err(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

const char *sep_error(void) { return g_err; }

/* ---- parameters --------------------------------------------------------- */
static kvlist g_par;
static char g_prog[256] = "swave";

static char *read_file(const char *path, size_t *len) {
  FILE *f = fopen(path, "rb");
  if (!f) return NULL;
  size_t cap = 1 << 16, n = 0;
  char *buf = (char *)malloc(cap + 1);
  size_t got;
  while ((got = fread(buf + n, 1, cap - n, f)) > 0) {
    n += got;
    if (n == cap) {
      cap *= 2;
      buf = (char *)realloc(buf, cap + 1);
    }
  }
  fclose(f);
  buf[n] = 0;
  *len = n;
  return buf;
}

int sep_init(int argc, char **argv) {
  kv_free(&g_par);
  if (argc > 0 && argv[0]) {
    const char *b = strrchr(argv[0], '/');
    snprintf(g_prog, sizeof(g_prog), "%s", b ? b + 1 : argv[0]);
  }
  for (int a = 1; a < argc; ++a) {
    const char *w = argv[a];
    const char *eq = strchr(w, '=');
    if (!eq || eq == w) continue;
    size_t vn = strlen(eq + 1);
    const char *v = eq + 1;
    if (vn >= 2 && (v[0] == '"' || v[0] == '\'') && v[vn - 1] == v[0]) {
      ++v;
      vn -= 2;
    }
    if ((size_t)(eq - w) == 3 && strncmp(w, "par", 3) == 0) {
      char path[4096];
      snprintf(path, sizeof(path), "%.*s", (int)vn, v);
      size_t len;
      char *text = read_file(path, &len);
      if (!text) {
        set_err("cannot read par file %s: %s", path, strerror(errno));
        return -1;
      }
      parse_pairs(text, len, &g_par);
      free(text);
      continue;
    }
    kv_add(&g_par, w, (size_t)(eq - w), v, vn);
  }
  return 0;
}

void sep_finish(void) { kv_free(&g_par); }

static int parse_int(const char *s, int *v) {
  char *end;
  errno = 0;
  const double d = strtod(s, &end); /* accepts 20, 20., 2e1 */
  if (end == s || errno) return -1;
  while (*end && isspace((unsigned char)*end)) ++end;
  if (*end) return -1;
  if (d != (double)(long)d) return -1;
  *v = (int)d;
  return 1;
}

static int parse_float(const char *s, float *v) {
  char *end;
  errno = 0;
  const double d = strtod(s, &end);
  if (end == s || errno) return -1;
  while (*end && isspace((unsigned char)*end)) ++end;
  if (*end) return -1;
  *v = (float)d;
  return 1;
}

static int parse_bool(const char *s, int *v) {
  char b[16];
  size_t n = 0;
  for (; s[n] && n < sizeof(b) - 1; ++n) b[n] = (char)tolower((unsigned char)s[n]);
  b[n] = 0;
  const char *yes[] = {"y", "yes", "t", "true", ".true.", "1"};
  const char *no[] = {"n", "no", "f", "false", ".false.", "0"};
  for (int i = 0; i < 6; ++i) {
    if (!strcmp(b, yes[i])) {
      *v = 1;
      return 1;
    }
    if (!strcmp(b, no[i])) {
      *v = 0;
      return 1;
    }
  }
  return -1;
}

static int get_str(const kvlist *l, const char *name, char *out, size_t n) {
  const char *s = kv_get(l, name);
  if (!s) return 0;
  snprintf(out, n, "%s", s);
  return 1;
}

int sep_par_str(const char *name, char *out, size_t n) { return get_str(&g_par, name, out, n); }
int sep_par_int(const char *name, int *v) {
  const char *s = kv_get(&g_par, name);
  return s ? parse_int(s, v) : 0;
}
int sep_par_float(const char *name, float *v) {
  const char *s = kv_get(&g_par, name);
  return s ? parse_float(s, v) : 0;
}
int sep_par_bool(const char *name, int *v) {
  const char *s = kv_get(&g_par, name);
  return s ? parse_bool(s, v) : 0;
}

int sep_exist(const char *tag) {
  if (!strcmp(tag, "in")) return kv_get(&g_par, "stdin") != NULL || !isatty(0);
  return kv_get(&g_par, tag) != NULL;
}

/* ---- datasets ----------------------------------------------------------- */
struct sep_file {
  int out;
  int big_endian;
  char tag[64];
  char hdr_path[4096];
  char bin_path[4096];
  kvlist hdr;   /* input header */
  kvlist puts;  /* output header values */
  FILE *bin;
  unsigned char *mem; /* samples embedded in a header read from standard input */
  size_t mem_len, mem_pos;
  char *hdr_mem;
};

static char *read_stream(FILE *f, size_t *len) {
  size_t cap = 1 << 16, n = 0;
  char *buf = (char *)malloc(cap + 1);
  size_t got;
  while ((got = fread(buf + n, 1, cap - n, f)) > 0) {
    n += got;
    if (n == cap) {
      cap *= 2;
      buf = (char *)realloc(buf, cap + 1);
    }
  }
  buf[n] = 0;
  *len = n;
  return buf;
}

static const char *find_marker(const char *buf, size_t len) {
  for (size_t i = 0; i + 1 < len; ++i)
    if (buf[i] == '\014' && buf[i + 1] == '\004') return buf + i;
  return NULL;
}

static int set_format(sep_file *f) {
  char fmt[64] = "xdr_float";
  get_str(&f->hdr, "data_format", fmt, sizeof(fmt));
  if (!strcmp(fmt, "xdr_float")) {
    f->big_endian = 1;
  } else if (!strcmp(fmt, "native_float")) {
    f->big_endian = 0;
  } else {
    set_err("%s: unsupported data_format \"%s\" (xdr_float or native_float)", f->hdr_path, fmt);
    return -1;
  }
  int esize = 4;
  if (sep_hdr_int(f, "esize", &esize) < 0 || esize != 4) {
    set_err("%s: esize must be 4", f->hdr_path);
    return -1;
  }
  return 0;
}

sep_file *sep_open_in(const char *tag) {
  sep_file *f = (sep_file *)calloc(1, sizeof(sep_file));
  snprintf(f->tag, sizeof(f->tag), "%s", tag);
  const char *path = kv_get(&g_par, !strcmp(tag, "in") ? "stdin" : tag);
  size_t len = 0;
  char *text;
  if (path) {
    snprintf(f->hdr_path, sizeof(f->hdr_path), "%s", path);
    text = read_file(path, &len);
    if (!text) {
      set_err("cannot read %s header %s: %s", tag, path, strerror(errno));
      free(f);
      return NULL;
    }
  } else if (!strcmp(tag, "in") && !isatty(0)) {
    snprintf(f->hdr_path, sizeof(f->hdr_path), "(standard input)");
    text = read_stream(stdin, &len);
  } else {
    set_err("no %s dataset: give %s=file.H", tag, !strcmp(tag, "in") ? "stdin" : tag);
    free(f);
    return NULL;
  }
  const char *mark = find_marker(text, len);
  const size_t hlen = mark ? (size_t)(mark - text) : len;
  parse_pairs(text, hlen, &f->hdr);
  char in[4096] = "";
  const int has_in = get_str(&f->hdr, "in", in, sizeof(in));
  if (!has_in || !strcmp(in, "stdin")) {
    if (!mark) {
      set_err("%s: no in= and no embedded samples", f->hdr_path);
      kv_free(&f->hdr);
      free(text);
      free(f);
      return NULL;
    }
    f->hdr_mem = text;
    f->mem = (unsigned char *)(mark + 2);
    f->mem_len = len - hlen - 2;
  } else {
    free(text);
    snprintf(f->bin_path, sizeof(f->bin_path), "%s", in);
    f->bin = fopen(in, "rb");
    if (!f->bin) {
      set_err("cannot open %s samples %s: %s", tag, in, strerror(errno));
      kv_free(&f->hdr);
      free(f);
      return NULL;
    }
  }
  if (set_format(f)) {
    sep_close(f);
    return NULL;
  }
  return f;
}

sep_file *sep_open_out(const char *tag) {
  const char *path = kv_get(&g_par, tag);
  if (!path) {
    set_err("no %s dataset: give %s=file.H", tag, tag);
    return NULL;
  }
  sep_file *f = (sep_file *)calloc(1, sizeof(sep_file));
  f->out = 1;
  f->big_endian = 1;
  snprintf(f->tag, sizeof(f->tag), "%s", tag);
  snprintf(f->hdr_path, sizeof(f->hdr_path), "%s", path);
  const char *dp = kv_get(&g_par, "datapath");
  if (!dp) dp = getenv("DATAPATH");
  if (dp && *dp) {
    const char *base = strrchr(path, '/');
    snprintf(f->bin_path, sizeof(f->bin_path), "%s%s%s@", dp,
             dp[strlen(dp) - 1] == '/' ? "" : "/", base ? base + 1 : path);
  } else {
    snprintf(f->bin_path, sizeof(f->bin_path), "%s@", path);
  }
  char fmt[64];
  if (sep_par_str("out_format", fmt, sizeof(fmt)) == 1 && !strcmp(fmt, "native_float"))
    f->big_endian = 0;
  f->bin = fopen(f->bin_path, "wb");
  if (!f->bin) {
    set_err("cannot create %s samples %s: %s", tag, f->bin_path, strerror(errno));
    free(f);
    return NULL;
  }
  return f;
}

int sep_hdr_str(const sep_file *f, const char *name, char *out, size_t n) {
  return get_str(&f->hdr, name, out, n);
}
int sep_hdr_int(const sep_file *f, const char *name, int *v) {
  const char *s = kv_get(&f->hdr, name);
  return s ? parse_int(s, v) : 0;
}
int sep_hdr_float(const sep_file *f, const char *name, float *v) {
  const char *s = kv_get(&f->hdr, name);
  return s ? parse_float(s, v) : 0;
}

static uint32_t load_u32(const unsigned char *b, int big) {
  return big ? ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | b[3]
             : ((uint32_t)b[3] << 24) | ((uint32_t)b[2] << 16) | ((uint32_t)b[1] << 8) | b[0];
}

static void store_u32(unsigned char *b, uint32_t u, int big) {
  if (big) {
    b[0] = (unsigned char)(u >> 24);
    b[1] = (unsigned char)(u >> 16);
    b[2] = (unsigned char)(u >> 8);
    b[3] = (unsigned char)u;
  } else {
    b[3] = (unsigned char)(u >> 24);
    b[2] = (unsigned char)(u >> 16);
    b[1] = (unsigned char)(u >> 8);
    b[0] = (unsigned char)u;
  }
}

enum { CHUNK = 1 << 16 };

int sep_read(sep_file *f, float *buf, size_t n) {
  if (f->out) {
    set_err("%s is an output dataset", f->tag);
    return -1;
  }
  unsigned char tmp[4 * 4096];
  size_t done = 0;
  while (done < n) {
    const size_t m = (n - done) < 4096 ? (n - done) : 4096;
    const unsigned char *src;
    if (f->mem) {
      if (f->mem_pos + 4 * m > f->mem_len) {
        set_err("%s: fewer samples than the header promises", f->hdr_path);
        return -1;
      }
      src = f->mem + f->mem_pos;
      f->mem_pos += 4 * m;
    } else {
      if (fread(tmp, 4, m, f->bin) != m) {
        set_err("%s: short read from %s", f->tag, f->bin_path);
        return -1;
      }
      src = tmp;
    }
    for (size_t i = 0; i < m; ++i) {
      const uint32_t u = load_u32(src + 4 * i, f->big_endian);
      memcpy(&buf[done + i], &u, 4);
    }
    done += m;
  }
  return 0;
}

int sep_write(sep_file *f, const float *buf, size_t n) {
  if (!f->out) {
    set_err("%s is an input dataset", f->tag);
    return -1;
  }
  unsigned char *tmp = (unsigned char *)malloc(4 * (size_t)CHUNK);
  size_t done = 0;
  while (done < n) {
    const size_t m = (n - done) < CHUNK ? (n - done) : CHUNK;
    for (size_t i = 0; i < m; ++i) {
      uint32_t u;
      memcpy(&u, &buf[done + i], 4);
      store_u32(tmp + 4 * i, u, f->big_endian);
    }
    if (fwrite(tmp, 4, m, f->bin) != m) {
      free(tmp);
      set_err("%s: write to %s failed", f->tag, f->bin_path);
      return -1;
    }
    done += m;
  }
  free(tmp);
  return 0;
}

int sep_put_str(sep_file *f, const char *name, const char *v) {
  kv_add(&f->puts, name, strlen(name), v, strlen(v));
  return 0;
}
int sep_put_int(sep_file *f, const char *name, int v) {
  char b[32];
  snprintf(b, sizeof(b), "%d", v);
  return sep_put_str(f, name, b);
}
int sep_put_float(sep_file *f, const char *name, float v) {
  char b[48];
  snprintf(b, sizeof(b), "%.9g", (double)v);
  return sep_put_str(f, name, b);
}

int sep_close(sep_file *f) {
  if (!f) return 0;
  int rc = 0;
  if (f->bin && fclose(f->bin)) rc = -1;
  if (f->out) {
    FILE *h = fopen(f->hdr_path, "w");
    if (!h) {
      set_err("cannot write header %s: %s", f->hdr_path, strerror(errno));
      rc = -1;
    } else {
      fprintf(h, "\n%s:\n", g_prog);
      fprintf(h, "\t\tin=\"%s\"\n", f->bin_path);
      fprintf(h, "\t\tesize=4\n");
      fprintf(h, "\t\tdata_format=\"%s\"\n", f->big_endian ? "xdr_float" : "native_float");
      for (size_t i = 0; i < f->puts.n; ++i) fprintf(h, "\t\t%s=%s\n", f->puts.k[i], f->puts.v[i]);
      if (fclose(h)) rc = -1;
    }
  }
  kv_free(&f->hdr);
  kv_free(&f->puts);
  free(f->hdr_mem);
  free(f);
  return rc;
}
