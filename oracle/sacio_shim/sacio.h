/* Minimal SAC I/O library interface (test infrastructure).
 *
 * Implements, from the published SAC binary file layout (header version 6:
 * 70 float words, 35 integer words, 5 logical words, 23 character fields of
 * 8 bytes with the 16-byte kevnm, then the samples; undefined values -12345),
 * the subset of the SAC library calls that the reference's CLI and reader use
 * (src/ReadManySacs.c, src/PCC_fullpair_1b.c): rsach, rsac1, get/set of float,
 * integer, character, logical and enumerated header variables, newhdr, wsac0.
 * Calling conventions follow the SAC library's C interface (names and string
 * lengths passed explicitly, error codes in *nerr).  Not thread safe: one
 * current header, as in the SAC library. */
#ifndef FPCC_SACIO_SHIM_H
#define FPCC_SACIO_SHIM_H

/* undefined header values */
#define SAC_FLOAT_UNDEFINED (-12345.0)
#define SAC_INT_UNDEFINED (-12345)
#define SAC_CHAR_UNDEFINED "-12345  "

#ifdef __cplusplus
extern "C" {
#endif

void rsach(char *kname, int *nerr, int kname_len);
void rsac1(char *kname, float *yarray, int *nlen, float *beg, float *del, int *max, int *nerr, int kname_len);
void getfhv(char *kname, float *fvalue, int *nerr, int kname_len);
void getnhv(char *kname, int *nvalue, int *nerr, int kname_len);
void getkhv(char *kname, char *kvalue, int *nerr, int kname_len, int kvalue_len);
void getlhv(char *kname, int *lvalue, int *nerr, int kname_len);
void setfhv(char *kname, float *fvalue, int *nerr, int kname_len);
void setnhv(char *kname, int *nvalue, int *nerr, int kname_len);
void setkhv(char *kname, char *kvalue, int *nerr, int kname_len, int kvalue_len);
void setlhv(char *kname, int *lvalue, int *nerr, int kname_len);
void setihv(char *kname, char *kvalue, int *nerr, int kname_len, int kvalue_len);
void newhdr(void);
void wsac0(char *kname, float *xarray, float *yarray, int *nerr, int kname_len);

#ifdef __cplusplus
}
#endif
#endif
