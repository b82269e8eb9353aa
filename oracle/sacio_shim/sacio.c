/* Minimal SAC I/O library (test infrastructure): see sacio.h.
 *
 * Header layout of a SAC binary file (version 6), as published with SAC:
 *   words   0-69   float variables (names in kFloat)
 *   words  70-104  integer variables, including the enumerated ones (kInt)
 *   words 105-109  logical variables (kLogical)
 *   bytes 440-631  character variables: kstnm (8), kevnm (16), then 21 x 8 (kChar)
 * followed by npts float samples.  Files are read in the host's byte order
 * (little-endian SAC files on little-endian hosts). */
#include "sacio.h"

#include <stdint.h>
#include <stdio.h>
#include <string.h>

#define SAC_UNDEF_F (-12345.0f)
#define SAC_UNDEF_I (-12345)
#define ERR_NOFILE 108
#define ERR_UNDEF 1336
#define ERR_NAME 1337
#define ERR_SHORT 801

static const char *kFloat[70] = {
    "delta", "depmin", "depmax", "scale", "odelta", "b", "e", "o", "a", "internal1",
    "t0", "t1", "t2", "t3", "t4", "t5", "t6", "t7", "t8", "t9",
    "f", "resp0", "resp1", "resp2", "resp3", "resp4", "resp5", "resp6", "resp7", "resp8",
    "resp9", "stla", "stlo", "stel", "stdp", "evla", "evlo", "evel", "evdp", "mag",
    "user0", "user1", "user2", "user3", "user4", "user5", "user6", "user7", "user8", "user9",
    "dist", "az", "baz", "gcarc", "internal2", "internal3", "depmen", "cmpaz", "cmpinc", "xminimum",
    "xmaximum", "yminimum", "ymaximum", "unused1", "unused2", "unused3", "unused4", "unused5", "unused6",
    "unused7"};
static const char *kInt[35] = {
    "nzyear", "nzjday", "nzhour", "nzmin", "nzsec", "nzmsec", "nvhdr", "norid", "nevid", "npts",
    "internal4", "nwfid", "nxsize", "nysize", "unused8", "iftype", "idep", "iztype", "unused9", "iinst",
    "istreg", "ievreg", "ievtyp", "iqual", "isynth", "imagtyp", "imagsrc", "unused10", "unused11", "unused12",
    "unused13", "unused14", "unused15", "unused16", "unused17"};
static const char *kLogical[5] = {"leven", "lpspol", "lovrok", "lcalda", "unused18"};
/* character variables: name, byte offset within the character block, length */
static const struct { const char *name; int off, len; } kChar[23] = {
    {"kstnm", 0, 8},    {"kevnm", 8, 16},   {"khole", 24, 8},   {"ko", 32, 8},      {"ka", 40, 8},
    {"kt0", 48, 8},     {"kt1", 56, 8},     {"kt2", 64, 8},     {"kt3", 72, 8},     {"kt4", 80, 8},
    {"kt5", 88, 8},     {"kt6", 96, 8},     {"kt7", 104, 8},    {"kt8", 112, 8},    {"kt9", 120, 8},
    {"kf", 128, 8},     {"kuser0", 136, 8}, {"kuser1", 144, 8}, {"kuser2", 152, 8}, {"kcmpnm", 160, 8},
    {"knetwk", 168, 8}, {"kdatrd", 176, 8}, {"kinst", 184, 8}};
/* enumerated values (the SAC list, in order from 1) */
static const char *kEnum[] = {
    "itime", "irlim", "iamph", "ixy", "iunkn", "idisp", "ivel", "iacc", "ib", "iday",
    "io", "ia", "it0", "it1", "it2", "it3", "it4", "it5", "it6", "it7", "it8", "it9"};

static struct {
  float f[70];
  int32_t i[35];
  int32_t l[5];
  char k[192];
} H;

/* name of length len (not necessarily terminated), compared case-insensitively */
static int name_eq(const char *a, int len, const char *b) {
  int n = 0;
  while (n < len && a[n] && a[n] != ' ') n++;
  if ((int)strlen(b) != n) return 0;
  for (int i = 0; i < n; i++) {
    char c = a[i];
    if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
    if (c != b[i]) return 0;
  }
  return 1;
}

static int find(const char **tab, int n, const char *name, int len) {
  for (int i = 0; i < n; i++)
    if (name_eq(name, len, tab[i])) return i;
  return -1;
}

static void cpath(char *dst, const char *src, int len) {
  int n = len < 1023 ? len : 1023;
  memcpy(dst, src, (size_t)n);
  dst[n] = '\0';
  while (n > 0 && dst[n - 1] == ' ') dst[--n] = '\0';
}

static int read_header(FILE *fp) {
  if (fread(H.f, 4, 70, fp) != 70 || fread(H.i, 4, 35, fp) != 35 || fread(H.l, 4, 5, fp) != 5 ||
      fread(H.k, 1, 192, fp) != 192)
    return ERR_SHORT;
  return 0;
}

void newhdr(void) {
  for (int i = 0; i < 70; i++) H.f[i] = SAC_UNDEF_F;
  for (int i = 0; i < 35; i++) H.i[i] = SAC_UNDEF_I;
  for (int i = 0; i < 5; i++) H.l[i] = 0;
  for (int i = 0; i < 23; i++) {
    memset(H.k + kChar[i].off, ' ', (size_t)kChar[i].len);
    memcpy(H.k + kChar[i].off, "-12345", 6);
  }
  H.i[6] = 6;    /* nvhdr */
  H.i[15] = 1;   /* iftype = itime */
  H.l[0] = 1;    /* leven */
}

void rsach(char *kname, int *nerr, int kname_len) {
  char path[1024];
  cpath(path, kname, kname_len);
  FILE *fp = fopen(path, "rb");
  if (!fp) { *nerr = ERR_NOFILE; return; }
  *nerr = read_header(fp);
  fclose(fp);
}

void rsac1(char *kname, float *yarray, int *nlen, float *beg, float *del, int *max, int *nerr, int kname_len) {
  char path[1024];
  cpath(path, kname, kname_len);
  FILE *fp = fopen(path, "rb");
  if (!fp) { *nerr = ERR_NOFILE; return; }
  *nerr = read_header(fp);
  if (!*nerr) {
    int n = H.i[9];
    if (n > *max) n = *max;
    if (n < 0) n = 0;
    if ((int)fread(yarray, 4, (size_t)n, fp) != n) *nerr = ERR_SHORT;
    *nlen = n;
    *beg = H.f[5];
    *del = H.f[0];
  }
  fclose(fp);
}

void getfhv(char *kname, float *fvalue, int *nerr, int kname_len) {
  const int k = find(kFloat, 70, kname, kname_len);
  if (k < 0) { *nerr = ERR_NAME; return; }
  *fvalue = H.f[k];
  *nerr = (H.f[k] == SAC_UNDEF_F) ? ERR_UNDEF : 0;
}

void getnhv(char *kname, int *nvalue, int *nerr, int kname_len) {
  const int k = find(kInt, 35, kname, kname_len);
  if (k < 0) { *nerr = ERR_NAME; return; }
  *nvalue = H.i[k];
  *nerr = (H.i[k] == SAC_UNDEF_I) ? ERR_UNDEF : 0;
}

void getlhv(char *kname, int *lvalue, int *nerr, int kname_len) {
  const int k = find(kLogical, 5, kname, kname_len);
  if (k < 0) { *nerr = ERR_NAME; return; }
  *lvalue = H.l[k];
  *nerr = 0;
}

void getkhv(char *kname, char *kvalue, int *nerr, int kname_len, int kvalue_len) {
  for (int i = 0; i < 23; i++) {
    if (!name_eq(kname, kname_len, kChar[i].name)) continue;
    const char *v = H.k + kChar[i].off;
    int n = kChar[i].len < kvalue_len ? kChar[i].len : kvalue_len;
    memcpy(kvalue, v, (size_t)n);
    while (n > 0 && (kvalue[n - 1] == ' ' || kvalue[n - 1] == '\0')) n--;
    kvalue[n] = '\0';
    *nerr = (strncmp(v, "-12345", 6) == 0) ? ERR_UNDEF : 0;
    return;
  }
  *nerr = ERR_NAME;
}

void setfhv(char *kname, float *fvalue, int *nerr, int kname_len) {
  const int k = find(kFloat, 70, kname, kname_len);
  if (k < 0) { *nerr = ERR_NAME; return; }
  H.f[k] = *fvalue;
  *nerr = 0;
}

void setnhv(char *kname, int *nvalue, int *nerr, int kname_len) {
  const int k = find(kInt, 35, kname, kname_len);
  if (k < 0) { *nerr = ERR_NAME; return; }
  H.i[k] = *nvalue;
  *nerr = 0;
}

void setlhv(char *kname, int *lvalue, int *nerr, int kname_len) {
  const int k = find(kLogical, 5, kname, kname_len);
  if (k < 0) { *nerr = ERR_NAME; return; }
  H.l[k] = *lvalue ? 1 : 0;
  *nerr = 0;
}

void setkhv(char *kname, char *kvalue, int *nerr, int kname_len, int kvalue_len) {
  for (int i = 0; i < 23; i++) {
    if (!name_eq(kname, kname_len, kChar[i].name)) continue;
    char *v = H.k + kChar[i].off;
    memset(v, ' ', (size_t)kChar[i].len);
    int n = kvalue_len < kChar[i].len ? kvalue_len : kChar[i].len;
    for (int j = 0; j < n && kvalue[j]; j++) v[j] = kvalue[j];
    *nerr = 0;
    return;
  }
  *nerr = ERR_NAME;
}

void setihv(char *kname, char *kvalue, int *nerr, int kname_len, int kvalue_len) {
  const int k = find(kInt, 35, kname, kname_len);
  if (k < 0) { *nerr = ERR_NAME; return; }
  const int e = find(kEnum, (int)(sizeof(kEnum) / sizeof(kEnum[0])), kvalue, kvalue_len);
  if (e < 0) { *nerr = ERR_NAME; return; }
  H.i[k] = e + 1;
  *nerr = 0;
}

void wsac0(char *kname, float *xarray, float *yarray, int *nerr, int kname_len) {
  (void)xarray;   /* evenly sampled data only */
  char path[1024];
  cpath(path, kname, kname_len);
  FILE *fp = fopen(path, "wb");
  if (!fp) { *nerr = ERR_NOFILE; return; }
  const int n = H.i[9] > 0 ? H.i[9] : 0;
  /* e, depmin, depmax, depmen from the samples as SAC writes them */
  if (n > 0 && H.f[0] != SAC_UNDEF_F && H.f[5] != SAC_UNDEF_F) H.f[6] = H.f[5] + (float)(n - 1) * H.f[0];
  if (n > 0) {
    float mn = yarray[0], mx = yarray[0];
    double s = 0;
    for (int j = 0; j < n; j++) {
      mn = yarray[j] < mn ? yarray[j] : mn;
      mx = yarray[j] > mx ? yarray[j] : mx;
      s += yarray[j];
    }
    H.f[1] = mn;
    H.f[2] = mx;
    H.f[56] = (float)(s / n);
  }
  int ok = fwrite(H.f, 4, 70, fp) == 70 && fwrite(H.i, 4, 35, fp) == 35 && fwrite(H.l, 4, 5, fp) == 5 &&
           fwrite(H.k, 1, 192, fp) == 192 && (int)fwrite(yarray, 4, (size_t)n, fp) == n;
  *nerr = ok ? 0 : ERR_SHORT;
  fclose(fp);
}
