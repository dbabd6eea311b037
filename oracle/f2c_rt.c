/*
 * f2c_rt.c -- runtime of the transliterated reference (oracle/_ref). TEST INFRASTRUCTURE ONLY:
 * linked only into oracle/_ref's libraries, which the tests and the CPU reference arm of the
 * benchmark use as the checker.
 */
#include "f2c_rt.h"

#include <ctype.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

jmp_buf f2c_stop_env;
static char g_stop_msg[256];

#define F2C_UNITS 100
static FILE* g_files[F2C_UNITS];

/* ---- captured formatted writes ---------------------------------------------------------- */
#define F2C_CAP_MAX (1 << 20)
typedef struct {
  int n;
  double written[F2C_CAP_MAX];
  double fp64[F2C_CAP_MAX];
} capture;
static capture* g_cap[F2C_UNITS];

void f2c_clear_captures(void) {
  for (int u = 0; u < F2C_UNITS; ++u)
    if (g_cap[u]) g_cap[u]->n = 0;
}

/* Copies up to max captured values of `unit` (written and FP64 operands); returns the count. */
int f2c_captured(int unit, double* written, double* fp64, int max) {
  if (unit < 0 || unit >= F2C_UNITS || !g_cap[unit]) return 0;
  const int n = g_cap[unit]->n < max ? g_cap[unit]->n : max;
  if (written) memcpy(written, g_cap[unit]->written, sizeof(double) * (size_t)n);
  if (fp64) memcpy(fp64, g_cap[unit]->fp64, sizeof(double) * (size_t)n);
  return g_cap[unit]->n;
}

const char* f2c_last_stop(void) { return g_stop_msg; }

void f2c_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int f2c_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void f2c_stop(const char* msg) {
  snprintf(g_stop_msg, sizeof g_stop_msg, "%s", msg);
  longjmp(f2c_stop_env, 1);
}

/* ---- units ---------------------------------------------------------------------------- */
static void trim(char* s) {
  size_t n = strlen(s);
  while (n && s[n - 1] == ' ') s[--n] = 0;
}

void f2c_open(int unit, const char* file, int formatted) {
  char name[512];
  snprintf(name, sizeof name, "%s", file);
  trim(name);
  if (unit < 0 || unit >= F2C_UNITS) f2c_stop("f2c_open: unit out of range");
  if (g_files[unit]) fclose(g_files[unit]);
  /* read-write without truncation: the reference opens inputs and outputs alike */
  FILE* f = fopen(name, formatted ? "r" : "rb");
  if (!f) f = fopen(name, formatted ? "w+" : "w+b");
  else {
    fclose(f);
    f = fopen(name, formatted ? "r+" : "r+b");
  }
  if (!f) f2c_stop("f2c_open: cannot open file");
  g_files[unit] = f;
}

void f2c_close(int unit) {
  if (unit >= 0 && unit < F2C_UNITS && g_files[unit]) {
    fclose(g_files[unit]);
    g_files[unit] = NULL;
  }
}

void f2c_flush(int unit) {
  if (unit >= 0 && unit < F2C_UNITS && g_files[unit]) fflush(g_files[unit]);
}

/* ---- list-directed read: values separated by blanks or commas, continuing over lines ---- */
static int next_value(FILE* f, char* buf, size_t cap) {
  int c;
  do {
    c = fgetc(f);
  } while (c != EOF && (isspace(c) || c == ','));
  if (c == EOF) return 0;
  size_t n = 0;
  while (c != EOF && !isspace(c) && c != ',') {
    if (n + 1 < cap) buf[n++] = (char)c;
    c = fgetc(f);
  }
  buf[n] = 0;
  /* a list-directed read statement consumes the rest of its last record */
  if (c == '\n') ungetc(c, f);
  return 1;
}

void f2c_read_list(int unit, const char* types, ...) {
  if (unit < 0 || unit >= F2C_UNITS || !g_files[unit]) f2c_stop("f2c_read_list: unit not open");
  FILE* f = g_files[unit];
  va_list ap;
  va_start(ap, types);
  char buf[128];
  for (const char* t = types; *t; ++t) {
    if (!next_value(f, buf, sizeof buf)) {
      va_end(ap);
      f2c_stop("f2c_read_list: end of file");
    }
    for (char* p = buf; *p; ++p)
      if (*p == 'd' || *p == 'D') *p = 'e'; /* Fortran exponent letter */
    switch (*t) {
      case 'i': *va_arg(ap, int*) = (int)strtol(buf, NULL, 10); break;
      case 'I': *va_arg(ap, long long*) = strtoll(buf, NULL, 10); break;
      case 'f': *va_arg(ap, float*) = strtof(buf, NULL); break;
      case 'd': *va_arg(ap, double*) = strtod(buf, NULL); break;
      default: break;
    }
  }
  va_end(ap);
  /* skip to the start of the next record */
  int c;
  while ((c = fgetc(f)) != EOF && c != '\n') {
  }
}

/* ---- unformatted sequential records: int32 length, data, int32 length ------------------ */
void f2c_read_unf(int unit, void* buf, long bytes) {
  if (unit < 0 || unit >= F2C_UNITS || !g_files[unit]) f2c_stop("f2c_read_unf: unit not open");
  FILE* f = g_files[unit];
  int32_t len = 0, len2 = 0;
  if (fread(&len, 4, 1, f) != 1) f2c_stop("f2c_read_unf: no record");
  if (len < bytes) f2c_stop("f2c_read_unf: record too short");
  if (fread(buf, 1, (size_t)bytes, f) != (size_t)bytes) f2c_stop("f2c_read_unf: short read");
  if (len > bytes) fseek(f, len - bytes, SEEK_CUR);
  if (fread(&len2, 4, 1, f) != 1 || len2 != len) f2c_stop("f2c_read_unf: bad record marker");
}

void f2c_write_unf(int unit, const void* buf, long bytes) {
  if (unit < 0 || unit >= F2C_UNITS || !g_files[unit]) f2c_stop("f2c_write_unf: unit not open");
  FILE* f = g_files[unit];
  const int32_t len = (int32_t)bytes;
  fwrite(&len, 4, 1, f);
  fwrite(buf, 1, (size_t)bytes, f);
  fwrite(&len, 4, 1, f);
}

void f2c_write_vals(int unit, int n, const double* written, const double* fp64) {
  if (unit < 0 || unit >= F2C_UNITS) return;
  if (!g_cap[unit]) {
    g_cap[unit] = (capture*)calloc(1, sizeof(capture));
    if (!g_cap[unit]) f2c_stop("f2c_write_vals: out of memory");
  }
  capture* c = g_cap[unit];
  for (int k = 0; k < n && c->n < F2C_CAP_MAX; ++k) {
    c->written[c->n] = written[k];
    c->fp64[c->n] = fp64[k];
    c->n++;
  }
}

/* ---- internal write: ('text', iW.M, ...) -------------------------------------------------- */
void f2c_write_internal(char* dst, int len, const char* fmt, int n, const long long* vals) {
  char out[512];
  size_t o = 0;
  int k = 0;
  const char* p = fmt;
  while (*p && o + 1 < sizeof out) {
    if (*p == '\'') {
      ++p;
      while (*p && o + 1 < sizeof out) {
        if (*p == '\'' && p[1] == '\'') {
          out[o++] = '\'';
          p += 2;
        } else if (*p == '\'') {
          ++p;
          break;
        } else {
          out[o++] = *p++;
        }
      }
    } else if ((*p == 'i' || *p == 'I') && isdigit((unsigned char)p[1])) {
      ++p;
      int w = (int)strtol(p, (char**)&p, 10), m = 1;
      if (*p == '.') {
        ++p;
        m = (int)strtol(p, (char**)&p, 10);
      }
      char num[64];
      snprintf(num, sizeof num, "%*.*lld", w, m, k < n ? vals[k] : 0LL);
      ++k;
      for (char* q = num; *q && o + 1 < sizeof out; ++q) out[o++] = *q;
    } else {
      ++p; /* parentheses, commas */
    }
  }
  out[o] = 0;
  /* a character variable is blank-padded to its length */
  int i = 0;
  for (; i < len && out[i]; ++i) dst[i] = out[i];
  for (; i < len; ++i) dst[i] = ' ';
  dst[len] = 0;
}

/* ---- arithmetic helpers -------------------------------------------------------------------- */
double f2c_powi_r8(double x, int n) {
  if (n < 0) return 1.0 / f2c_powi_r8(x, -n);
  double r = 1.0;
  for (int k = 0; k < n; ++k) r = (k == 0) ? x : r * x;
  return n == 0 ? 1.0 : r;
}

float f2c_powi_r4(float x, int n) {
  if (n < 0) return 1.0f / f2c_powi_r4(x, -n);
  float r = 1.0f;
  for (int k = 0; k < n; ++k) r = (k == 0) ? x : r * x;
  return n == 0 ? 1.0f : r;
}

int f2c_powi_i4(int x, int n) {
  int r = 1;
  for (int k = 0; k < n; ++k) r *= x;
  return r;
}

double f2c_sum_r8(const double* a, long lo, long hi) {
  double s = 0.0;
  for (long k = lo; k <= hi; ++k) s += a[k - 1];
  return s;
}

float f2c_sum_r4(const float* a, long lo, long hi) {
  float s = 0.0f;
  for (long k = lo; k <= hi; ++k) s += a[k - 1];
  return s;
}

int cudamemgetinfo(void* fre, void* tot) {
  *(long long*)fre = 0;
  *(long long*)tot = 0;
  return 0;
}
