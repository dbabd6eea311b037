/*
 * f2c_rt.h -- runtime of the transliterated reference (oracle/_ref). TEST INFRASTRUCTURE ONLY.
 *
 * The C that oracle/f2c_ref.py generates from the reference's Fortran calls these for what the
 * Fortran runtime did: units opened by number, list-directed and unformatted sequential I/O
 * (4-byte record markers, the format of the reference's fields/w.NNN files), internal writes
 * that build file names, STOP, and integer powers. Formatted writes to numbered units (the
 * spectra, fluxes and budgets of src/diagnostics.f90) are captured in memory for the tests.
 */
#ifndef F2C_RT_H
#define F2C_RT_H

#include <setjmp.h>

#ifdef __cplusplus
extern "C" {
#endif

extern jmp_buf f2c_stop_env;

void f2c_open(int unit, const char* file, int formatted);
void f2c_close(int unit);
void f2c_flush(int unit);
/* list-directed read: types is one letter per item ('i' int, 'I' long long, 'f' float,
 * 'd' double), each followed by a pointer */
void f2c_read_list(int unit, const char* types, ...);
void f2c_read_unf(int unit, void* buf, long bytes);
void f2c_write_unf(int unit, const void* buf, long bytes);
/* formatted write of n values to a numbered unit: captured (written values, and the FP64
 * operand of a real() conversion) */
void f2c_write_vals(int unit, int n, const double* written, const double* fp64);
/* internal write of integers into a character variable with a format of quoted strings and
 * iW.M edit descriptors */
void f2c_write_internal(char* dst, int len, const char* fmt, int n, const long long* vals);
void f2c_stop(const char* msg);

double f2c_powi_r8(double x, int n);
float f2c_powi_r4(float x, int n);
int f2c_powi_i4(int x, int n);
double f2c_sum_r8(const double* a, long lo, long hi);
float f2c_sum_r4(const float* a, long lo, long hi);

/* stub of the CUDA call in show_mem (trunc.f90): reports zero bytes */
int cudamemgetinfo(void* fre, void* tot);

/* cuFFT shim (cufft_shim.c) */
int cufftexecd2z(int plan, void* idata, void* odata);
int cufftexecz2d(int plan, void* idata, void* odata);

#ifdef __cplusplus
}
#endif

#endif
