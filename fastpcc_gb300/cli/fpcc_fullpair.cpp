// fpcc_fullpair: interstation correlations of two stations' records on the GPU,
// with the argv grammar of the reference CLI (src/PCC_fullpair_1b.c:146-196):
//
//   fpcc_fullpair filelist1 filelist2 [pcc] [v=] [wpcc] [ccgn] [cc1b] [tl1= tl2= | nl1= nl2=]
//                 [isac | imsacs] [osac | obin[=prefix]] [clip] [std=] [awhite=f1,f2]
//                 [mindist=] [maxdist=] [pmin= pmax= VR= V= type= w0=] [Nmax=] [mincc=]
//                 [NoAutoPairing] [verbose=] [stack=lin,pws,tspws] [nu=]
//
// Records are SAC files listed one per line (isac) or MSACS1 files (imsacs).
// The steps follow the reference's order (PCCfullpair_main :211-521): read both
// stations, drop all-zero traces, drop traces whose rms exceeds std times the
// median rms, clip, sort by start time and keep the times present at both
// stations (or pair line by line), whiten, flip reversed components, then
// correlate with each requested method and write one SAC file per window pair
// (osac) or one binary file per channel pair (obin, the ts-PWS input format).
// With stack=, the windows of each channel pair are also stacked on the device
// (linear, phase-weighted, time-scale phase-weighted; fpcc_stack, coherence
// power nu=, the ts-PWS wavelet family from pmin= pmax= V= type= w0= as for
// WPCC) and each stack is written as one SAC file, <pair>_<method>_<kind>.sac.
//
// GPU side: the record files are read by a pool of threads straight into
// pinned memory and the kept windows uploaded asynchronously; clipping and
// whitening run on the device (fpcc_clip_rows, fpcc_whiten_rows); every method
// then runs one station stage and one pair stage over all windows
// (fpcc_station_stage, fpcc_pair_stage, WPCC plans), and a thread pool writes
// the output files.  PCC at powers other than 1 and 2 uses the normalisation
// 2(N - |lag|) of the reference's CUDA build (src/ccs_cuda.cu:452).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fastpcc_gb300.h"

namespace {

// ------------------------------------------------------------------ records
// Trace metadata; the MSACS1 file format stores exactly this record per trace
// (src/ReadManySacs.h:7-30), so its layout is kept.
struct TraceHeader {
  int32_t npts;
  float dt, b;
  int32_t year, yday, hour, min, sec, msec;
  time_t t;
  float stla, stlo, stel, stdp, cmpaz, cmpinc;
  char sta[9], net[9], chn[9], loc[9];
  int32_t nostloc, nocmp;
};
static_assert(sizeof(time_t) == 8, "MSACS1 records hold an 8-byte time_t");
static_assert(sizeof(TraceHeader) == 120, "MSACS1 record layout");

struct MsacsHeader {   // src/ReadManySacs.h:32-37
  char FormatID[8];
  int32_t nseq, npts, SingleChannel;
};

struct CcHeader {      // the obin header (src/sac2bin.h:6-27)
  char method[8], net1[8], sta1[8], loc1[8], chn1[8], net2[8], sta2[8], loc2[8], chn2[8];
  float stlat1, stlon1, stel1, stlat2, stlon2, stel2;
  uint32_t nlags, nseq;
  float tlength, lag1, lag2;
};

constexpr float kUndefF = -12345.0f;
constexpr int kUndefI = -12345;

// Days since 1970 with the proleptic Gregorian leap rule, day of year from 1.
time_t utc_seconds(int year, int yday, int hour, int min, int sec) {
  auto leap = [](int y) { return (y % 4) == 0 && ((y % 100) != 0 || (y % 400) == 0); };
  long long d = 0;
  for (int y = 1970; y < year; y++) d += leap(y) ? 366 : 365;
  d += yday - 1;
  return (time_t)(((d * 24 + hour) * 60 + min) * 60 + sec);
}

// One SAC header field of 8 characters: cut at the first blank, "-12345" is undefined.
void sac_string(const char* src, char* dst) {
  memset(dst, 0, 9);
  memcpy(dst, src, 8);
  if (char* p = (char*)memchr(dst, ' ', 8)) *p = '\0';
  if (!strncmp(dst, "-12345", 6)) dst[0] = '\0';
}

// Reads the SAC file header and up to maxn samples (little-endian SAC v6 layout:
// 70 floats, 35 integers, 5 logicals, 192 bytes of character fields, samples).
bool read_sac(const std::string& path, TraceHeader& h, float* data, int maxn, int* npts_file) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  float fh[70];
  int32_t ih[40];
  char kh[192];
  bool ok = fread(fh, 4, 70, f) == 70 && fread(ih, 4, 40, f) == 40 && fread(kh, 1, 192, f) == 192;
  if (ok) {
    memset(&h, 0, sizeof h);
    const int npts = ih[9];
    *npts_file = npts;
    h.npts = npts;
    h.dt = fh[0];
    h.b = fh[5];
    h.year = ih[0]; h.yday = ih[1]; h.hour = ih[2]; h.min = ih[3]; h.sec = ih[4]; h.msec = ih[5];
    sac_string(kh + 0, h.sta);
    sac_string(kh + 24, h.loc);
    sac_string(kh + 160, h.chn);
    sac_string(kh + 168, h.net);
    h.stla = fh[31]; h.stlo = fh[32];
    if (h.stla == kUndefF || h.stlo == kUndefF) h.nostloc = 1;
    h.stel = fh[33] == kUndefF ? 0.f : fh[33];
    h.stdp = fh[34] == kUndefF ? 0.f : fh[34];
    h.cmpaz = fh[57]; h.cmpinc = fh[58];
    if (h.cmpaz == kUndefF || h.cmpinc == kUndefF) h.nocmp = 1;
    h.t = utc_seconds(h.year, h.yday, h.hour, h.min, h.sec);
    if (data) {
      const int n = std::max(0, std::min(npts, maxn));
      ok = (int)fread(data, 4, (size_t)n, f) == n;
    }
  }
  fclose(f);
  return ok;
}

bool write_sac(const std::string& path, const float* y, int n, float b, float dt, const char* kinst,
               const TraceHeader& h1, const TraceHeader& h2) {
  float fh[70];
  int32_t ih[40];
  char kh[192];
  for (float& v : fh) v = kUndefF;
  for (int i = 0; i < 35; i++) ih[i] = kUndefI;
  for (int i = 35; i < 40; i++) ih[i] = 0;
  // character fields undefined: kstnm (8 bytes), kevnm (16), then 21 fields of 8
  memset(kh, ' ', 192);
  for (int off = 0; off < 192; off += (off == 8 ? 16 : 8)) memcpy(kh + off, "-12345", 6);
  auto kset = [&](int off, int len, const char* v) {
    memset(kh + off, ' ', len);
    memcpy(kh + off, v, std::min<size_t>(strlen(v), 8));
  };
  ih[6] = 6;     // nvhdr
  ih[15] = 1;    // iftype: time series
  ih[35] = 1;    // leven
  ih[9] = n;
  fh[0] = dt;
  kset(184, 8, kinst);
  if (!h1.nostloc && !h2.nostloc) {
    fh[31] = h2.stla; fh[32] = h2.stlo; fh[33] = h2.stel; fh[34] = h2.stdp;
    kset(168, 8, h2.net); kset(0, 8, h2.sta); kset(24, 8, h2.loc); kset(160, 8, h2.chn);
    fh[35] = h1.stla; fh[36] = h1.stlo; fh[37] = h1.stel; fh[38] = h1.stdp;
    kset(136, 8, h1.net); kset(8, 16, h1.sta); kset(144, 8, h1.loc); kset(152, 8, h1.chn);
  }
  ih[38] = 1;    // lcalda
  ih[0] = h1.year; ih[1] = h1.yday; ih[2] = h1.hour; ih[3] = h1.min; ih[4] = h1.sec; ih[5] = h1.msec;
  const float lag0 = (float)(difftime(h1.t, h2.t) + (double)(h1.msec - h2.msec) / 1000 + (h1.b - h2.b));
  fh[5] = b;
  fh[7] = lag0;
  kset(32, 8, "0LagTime");
  ih[17] = 11;   // iztype: origin time
  if (n > 0) {
    float mn = y[0], mx = y[0];
    double s = 0;
    for (int i = 0; i < n; i++) { mn = std::min(mn, y[i]); mx = std::max(mx, y[i]); s += y[i]; }
    fh[1] = mn; fh[2] = mx; fh[56] = (float)(s / n);
    fh[6] = b + (float)(n - 1) * dt;
  }
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = fwrite(fh, 4, 70, f) == 70 && fwrite(ih, 4, 40, f) == 40 && fwrite(kh, 1, 192, f) == 192 &&
            (int)fwrite(y, 4, (size_t)n, f) == n;
  return fclose(f) == 0 && ok;
}

// ------------------------------------------------------------------ options
struct Options {
  double tl1 = 0, tl2 = 0, v = 2;
  int nl1 = 0, nl2 = 0;
  int iformat = 1, oformat = 1;
  int pcc = 0, wpcc = 0, ccgn = 0, cc1b = 0, clip = 0;
  int mincc = 0, Nmax = 0;
  double stdn = 0, mindist = 0, maxdist = 0, pmin = 0, pmax = 0, VR = 0;
  unsigned V = 2;
  int type = -3;
  double op1 = 0;
  double awhite[2] = {0, 0};
  std::string fin1, fin2, obinprefix;
  bool has_prefix = false;
  int autopair = 1, acc = 0, verbose = 1;
  int stack = 0;      // bit 0 linear, bit 1 PWS, bit 2 ts-PWS
  double nu = 2;
};

bool rd_double(double* x, const char* s) { char* e; *x = strtod(s, &e); return e != s; }
bool rd_int(int* x, const char* s) { char* e; *x = (int)strtol(s, &e, 10); return e != s; }

int parse(int argc, char** argv, Options& o) {
  o.fin1 = argv[1];
  o.fin2 = argv[2];
  o.acc = (o.fin1 == o.fin2) ? 1 : 0;
  int er = 0;
  for (int i = 1; i < argc; i++) {
    const char* a = argv[i];
    auto is = [&](const char* k) { return !strncmp(a, k, strlen(k)); };
    int iv;
    if (is("tl1=")) er += !rd_double(&o.tl1, a + 4);
    else if (is("tl2=")) er += !rd_double(&o.tl2, a + 4);
    else if (is("v=")) er += !rd_double(&o.v, a + 2);
    else if (is("nl1=")) er += !rd_int(&o.nl1, a + 4);
    else if (is("nl2=")) er += !rd_int(&o.nl2, a + 4);
    else if (is("isac")) o.iformat = 1;
    else if (is("imsacs")) o.iformat = 2;
    else if (is("osac")) o.oformat = 1;
    else if (is("obin")) {
      o.oformat = 2;
      if (is("obin=")) { o.obinprefix = a + 5; o.has_prefix = true; }
    } else if (is("pcc")) o.pcc = 1;
    else if (is("wpcc")) o.wpcc = 1;
    else if (is("ccgn")) o.ccgn = 1;
    else if (is("cc1b")) o.cc1b = 1;
    else if (is("clip")) o.clip = 1;
    else if (is("std=")) er += !rd_double(&o.stdn, a + 4);
    else if (is("mindist=")) er += !rd_double(&o.mindist, a + 8);
    else if (is("maxdist=")) er += !rd_double(&o.maxdist, a + 8);
    else if (is("pmin=")) er += !rd_double(&o.pmin, a + 5);
    else if (is("pmax=")) er += !rd_double(&o.pmax, a + 5);
    else if (is("VR=")) er += !rd_double(&o.VR, a + 3);
    else if (is("mincc=")) er += !rd_int(&o.mincc, a + 6);
    else if (is("Nmax=")) er += !rd_int(&o.Nmax, a + 5);
    else if (is("V=")) { er += !rd_int(&iv, a + 2); o.V = (unsigned)iv; }
    else if (is("type=")) er += !rd_int(&o.type, a + 5);
    else if (is("w0=")) er += !rd_double(&o.op1, a + 3);
    else if (is("awhite=")) {
      if (sscanf(a + 7, "%lf,%lf", &o.awhite[0], &o.awhite[1]) != 2) er++;
    } else if (is("stack=")) {
      std::string v = a + 6;
      size_t p0 = 0;
      while (p0 <= v.size()) {
        size_t p1 = v.find(',', p0);
        if (p1 == std::string::npos) p1 = v.size();
        const std::string k = v.substr(p0, p1 - p0);
        if (k == "lin") o.stack |= 1;
        else if (k == "pws") o.stack |= 2;
        else if (k == "tspws") o.stack |= 4;
        else er++;
        p0 = p1 + 1;
      }
    } else if (is("nu=")) er += !rd_double(&o.nu, a + 3);
    else if (is("NoAutoPairing")) o.autopair = 0;
    else if (is("verbose=")) er += !rd_int(&o.verbose, a + 8);
  }
  if (!o.autopair && o.stdn > 0) {
    printf("fpcc_fullpair: Warning, the std option cannot be used without automatic trace pairing.\n");
    o.stdn = 0;
  }
  if (o.pmin > o.pmax) {
    printf("fpcc_fullpair: Error, pmax has to be higher than pmin.\n");
    er++;
  }
  return er;
}

// ------------------------------------------------------------------ reading
struct Station {
  std::vector<TraceHeader> hdr;
  float* x = nullptr;        // Tr x N, pinned when the CUDA driver allows it
  bool pinned = false;
  int N = 0, Tr = 0;
  float dt = 0;
};

// Page-locked host memory for the traces (faster, asynchronous uploads); plain
// memory where no device is reachable yet, so that reading and pairing still run.
float* host_alloc(size_t n, bool* pinned) {
  float* p = nullptr;
  *pinned = cudaMallocHost(&p, n * sizeof(float)) == cudaSuccess;
  if (!*pinned) {
    cudaGetLastError();
    p = (float*)malloc(n * sizeof(float));
  }
  if (p) memset(p, 0, n * sizeof(float));
  return p;
}

void host_free(float* p, bool pinned) {
  if (pinned) cudaFreeHost(p);
  else free(p);
}

std::vector<std::string> read_list(const std::string& path) {
  std::vector<std::string> v;
  FILE* f = fopen(path.c_str(), "r");
  if (!f) return v;
  char line[1024];
  while (fgets(line, sizeof line, f)) {
    if (char* p = strchr(line, '\n')) *p = '\0';
    v.emplace_back(line);
  }
  fclose(f);
  return v;
}

void parallel_for(int n, const std::function<void(int)>& fn) {
  const int nt = std::max(1, std::min(n, (int)std::thread::hardware_concurrency()));
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++)
    th.emplace_back([&] {
      for (int i; (i = next++) < n;) fn(i);
    });
  for (auto& t : th) t.join();
}

// SAC list: the first file sets N (or Nmax), dt and b; shorter traces, other
// sampling intervals or begin times are skipped, longer ones cut
// (src/ReadManySacs.c:161-323).  Files are read in parallel into pinned memory.
int read_sac_station(const std::string& list, int Nmax, Station& st) {
  const std::vector<std::string> files = read_list(list);
  if (files.empty()) { printf("fpcc_fullpair: nothing to read in %s\n", list.c_str()); return -2; }
  TraceHeader h0;
  int npts0 = 0;
  if (!read_sac(files[0], h0, nullptr, 0, &npts0)) { printf("fpcc_fullpair: cannot read %s\n", files[0].c_str()); return -2; }
  const int N = Nmax > 0 ? Nmax : npts0;
  const float dt1 = h0.dt, b1 = h0.b;
  const int Tr = (int)files.size();
  bool pinned = false;
  float* x = host_alloc((size_t)Tr * N, &pinned);
  if (!x) { printf("fpcc_fullpair: out of host memory\n"); return 4; }
  std::vector<TraceHeader> hdr(Tr);
  std::vector<int> keep(Tr, 0);
  std::atomic<int> bad{0};
  parallel_for(Tr, [&](int i) {
    int npts = 0;
    if (!read_sac(files[i], hdr[i], x + (size_t)i * N, N, &npts)) { bad = i + 1; return; }
    if (npts < N) return;                                       // too short: skipped
    if (std::fabs(hdr[i].dt - dt1) > dt1 * 0.001) return;       // other sampling interval
    if (std::fabs(b1 - hdr[i].b) > dt1) return;                 // other begin time
    if (npts > N) hdr[i].npts = N;
    keep[i] = 1;
  });
  if (bad) { printf("fpcc_fullpair: error reading %s\n", files[bad - 1].c_str()); host_free(x, pinned); return -2; }
  int k = 0;
  for (int i = 0; i < Tr; i++) {
    if (!keep[i]) {
      printf("fpcc_fullpair: skipping %s (length, sampling or begin time differ from the first file)\n",
             files[i].c_str());
      continue;
    }
    if (k != i) memmove(x + (size_t)k * N, x + (size_t)i * N, (size_t)N * sizeof(float));
    hdr[k++] = hdr[i];
  }
  hdr.resize(k);
  st.hdr = hdr;
  st.x = x;
  st.pinned = pinned;
  st.N = N;
  st.Tr = k;
  st.dt = dt1;
  return 0;
}

// MSACS1 file: a 20-byte header, then per trace one metadata record and npts samples.
int read_msacs_station(const std::string& path, Station& st) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) { printf("fpcc_fullpair: cannot open %s\n", path.c_str()); return -2; }
  MsacsHeader mh;
  if (fread(&mh, sizeof mh, 1, f) != 1 || strcmp(mh.FormatID, "MSACS1") || mh.npts == 0) {
    printf("fpcc_fullpair: %s is not an MSACS1 file of equal-length traces\n", path.c_str());
    fclose(f);
    return -2;
  }
  const int Tr = mh.nseq, N = mh.npts;
  bool pinned = false;
  float* x = host_alloc((size_t)Tr * N, &pinned);
  if (!x) { fclose(f); printf("fpcc_fullpair: out of host memory\n"); return 4; }
  std::vector<TraceHeader> hdr(Tr);
  for (int i = 0; i < Tr; i++) {
    int n;
    if (fread(&hdr[i], sizeof(TraceHeader), 1, f) != 1 ||
        (int)fread(x + (size_t)i * N, 4, (size_t)(n = std::min(N, hdr[i].npts)), f) != n) {
      printf("fpcc_fullpair: unexpected end of %s\n", path.c_str());
      fclose(f);
      host_free(x, pinned);
      return 5;
    }
  }
  fclose(f);
  st.hdr = hdr;
  st.x = x;
  st.pinned = pinned;
  st.N = N;
  st.Tr = Tr;
  st.dt = Tr ? hdr[0].dt : 0.f;
  return 0;
}

// ------------------------------------------------------------------ selection
float median_of(std::vector<float> a) {   // the mean of the two middle values for even counts
  if (a.empty()) return 0.f;
  const size_t k = a.size() / 2;
  std::nth_element(a.begin(), a.begin() + k, a.end());
  float m = a[k];
  if (a.size() % 2 == 0) m = (m + *std::max_element(a.begin(), a.begin() + k)) / 2;
  return m;
}

// Indices of the traces kept, in the station's order.
std::vector<int> select_traces(const Station& st, double stdn) {
  std::vector<int> idx;
  for (int i = 0; i < st.Tr; i++) {
    const float* r = st.x + (size_t)i * st.N;
    bool nz = false;
    for (int n = 0; n < st.N && !nz; n++) nz = r[n] != 0;
    if (nz) idx.push_back(i);
    else printf("fpcc_fullpair: skipping %s.%s.%s.%s at %4d-%03d %02d:%02d:%02d, all zeros\n", st.hdr[i].net,
                st.hdr[i].sta, st.hdr[i].loc, st.hdr[i].chn, st.hdr[i].year, st.hdr[i].yday, st.hdr[i].hour,
                st.hdr[i].min, st.hdr[i].sec);
  }
  if (stdn > 0) {
    std::vector<float> sd(idx.size());
    for (size_t j = 0; j < idx.size(); j++) {
      const float* r = st.x + (size_t)idx[j] * st.N;
      double s = 0;
      for (int n = 0; n < st.N; n++) s += (double)r[n] * r[n];
      sd[j] = (float)std::sqrt(s / st.N);
    }
    const float med = median_of(sd);
    std::vector<int> kept;
    for (size_t j = 0; j < idx.size(); j++) {
      if (sd[j] > stdn * med) printf("fpcc_fullpair: skipping sequence %d, its std is %f times the median std\n",
                                     idx[j], sd[j] / med);
      else kept.push_back(idx[j]);
    }
    idx = kept;
  }
  return idx;
}

double tdiff(const TraceHeader& a, const TraceHeader& b) {
  return difftime(a.t, b.t) + (double)(a.msec - b.msec) / 1000;
}

void sort_by_time(const Station& st, std::vector<int>& idx) {
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return (int)tdiff(st.hdr[a], st.hdr[b]) < 0; });
}

// Times present at both stations (within half a second), in time order.
void pair_lists(const Station& s1, std::vector<int>& i1, const Station& s2, std::vector<int>& i2) {
  std::vector<int> o1, o2;
  size_t a = 0, b = 0;
  while (a < i1.size() && b < i2.size()) {
    const double td = tdiff(s1.hdr[i1[a]], s2.hdr[i2[b]]);
    if (std::fabs(td) < 0.5) { o1.push_back(i1[a++]); o2.push_back(i2[b++]); }
    else if (td < 0) a++;
    else b++;
  }
  i1 = o1;
  i2 = o2;
}

// ------------------------------------------------------------------ output
void store_sacs(const std::vector<float>& y, int L, int Tr, int Lag1, const std::vector<TraceHeader>& h1,
                const std::vector<TraceHeader>& h2, float dt, const char* name) {
  parallel_for(Tr, [&](int t) {
    const TraceHeader &a = h1[t], &b = h2[t];
    char fn[160];
    snprintf(fn, sizeof fn, "%s.%s.%s.%s.%s.%s.%s.%s_%s_%04d.%03d.%02d.%02d.%02d.sac", a.net, a.sta, a.loc, a.chn,
             b.net, b.sta, b.loc, b.chn, name, a.year, a.yday, a.hour, a.min, a.sec);
    if (!write_sac(fn, y.data() + (size_t)t * L, L, Lag1 * dt, dt, name, a, b))
      printf("fpcc_fullpair: error writing %s\n", fn);
  });
}

// One file per (channel 1, channel 2) set (src/PCC_fullpair_1b.c:761-829): header,
// the start times, the zero-lag offsets, the correlations.
void store_bins(const std::vector<float>& y, int L, int Tr, int Lag1, const std::vector<TraceHeader>& h1,
                const std::vector<TraceHeader>& h2, float dt, const char* name, const Options& o) {
  std::vector<char> done(Tr + 1, 0);
  int next = 0;
  while (next < Tr) {
    std::vector<int> set;
    for (int t = 0; t < Tr; t++)
      if (!strcmp(h1[t].chn, h1[next].chn) && !strcmp(h2[t].chn, h2[next].chn)) { done[t] = 1; set.push_back(t); }
    const TraceHeader &a = h1[set[0]], &b = h2[set[0]];
    char fn[160];
    if (o.has_prefix)
      snprintf(fn, sizeof fn, "%s.%s.%s%c.%s.%s%c_%s.bin", o.obinprefix.c_str(), a.sta, a.loc, a.chn[2], b.sta, b.loc,
               b.chn[2], name);
    else
      snprintf(fn, sizeof fn, "%s.%s%c.%s.%s%c_%s.bin", a.sta, a.loc, a.chn[2], b.sta, b.loc, b.chn[2], name);
    CcHeader ch;
    memset(&ch, 0, sizeof ch);
    strncpy(ch.method, name, 8);
    memcpy(ch.net1, a.net, 8); memcpy(ch.sta1, a.sta, 8); memcpy(ch.loc1, a.loc, 8); memcpy(ch.chn1, a.chn, 8);
    memcpy(ch.net2, b.net, 8); memcpy(ch.sta2, b.sta, 8); memcpy(ch.loc2, b.loc, 8); memcpy(ch.chn2, b.chn, 8);
    ch.stlat1 = a.stla; ch.stlon1 = a.stlo; ch.stel1 = a.stel;
    ch.stlat2 = b.stla; ch.stlon2 = b.stlo; ch.stel2 = b.stel;
    ch.nlags = (uint32_t)L;
    ch.nseq = (uint32_t)set.size();
    ch.tlength = dt * (L - 1);
    ch.lag1 = dt * Lag1;
    ch.lag2 = dt * (Lag1 + L - 1);
    std::vector<time_t> tt(set.size());
    for (size_t j = 0; j < set.size(); j++) tt[j] = h1[set[j]].t;
    // the reference takes the offset of the set's last station-1 record against
    // its first station-2 record for every entry (src/PCC_fullpair_1b.c:735-738)
    const TraceHeader &la = h1[set.back()], &fb = h2[set[0]];
    const float off = (float)(tdiff(la, fb) + (la.b - fb.b));
    std::vector<float> lag0(set.size(), off);
    FILE* f = fopen(fn, "wb");
    if (!f) { printf("fpcc_fullpair: cannot create %s\n", fn); }
    else {
      fwrite(&ch, sizeof ch, 1, f);
      fwrite(tt.data(), sizeof(time_t), tt.size(), f);
      fwrite(lag0.data(), sizeof(float), lag0.size(), f);
      for (int t : set) fwrite(y.data() + (size_t)t * L, sizeof(float), (size_t)L, f);
      fclose(f);
    }
    while (done[next]) next++;
  }
}

// ------------------------------------------------------------------ GPU
#define GCHECK(call)                                                                               \
  do {                                                                                             \
    const int rc_ = (call);                                                                        \
    if (rc_) { printf("fpcc_fullpair: %s failed (%d): %s\n", #call, rc_, fpcc_last_error()); return rc_; } \
  } while (0)

double gcarc_deg(double lat1, double lon1, double lat2, double lon2) {
  const double d2r = 3.14159265358979323846 / 180.0;
  lat1 *= d2r; lon1 *= d2r; lat2 *= d2r; lon2 *= d2r;
  double s = std::sin((lon1 - lon2) / 2);
  s *= s;
  const double c = std::cos(lat2 - lat1) * (1 - s) - std::cos(lat2 + lat1) * s;
  return std::acos(std::max(-1.0, std::min(1.0, c))) / d2r;
}

int run(const Options& o) {
  Station s1, s2;
  int rc = (o.iformat == 2) ? read_msacs_station(o.fin1, s1) : read_sac_station(o.fin1, o.Nmax, s1);
  if (rc) return rc;
  if (!o.acc) {
    rc = (o.iformat == 2) ? read_msacs_station(o.fin2, s2) : read_sac_station(o.fin2, o.Nmax, s2);
    if (rc) return rc;
  }
  const Station& t2 = o.acc ? s1 : s2;
  const int N = s1.N;
  if (!o.acc && s2.N != N) printf("fpcc_fullpair: These traces have different lengths: %d:%d\n", N, s2.N);
  const float dt = t2.dt;
  // station locations (first record) and the distance gates
  bool stloc = s1.Tr > 0 && !s1.hdr[0].nostloc && t2.Tr > 0 && !t2.hdr[0].nostloc;
  double gcarc = 0;
  Options opt = o;
  if (stloc) {
    gcarc = gcarc_deg(s1.hdr[0].stla, s1.hdr[0].stlo, t2.hdr[0].stla, t2.hdr[0].stlo);
    if (opt.mindist > 0 && gcarc < opt.mindist) { printf("fpcc_fullpair: the stations are closer than %f degrees\n", opt.mindist); return 0; }
    if (opt.maxdist > 0 && gcarc > opt.maxdist) { printf("fpcc_fullpair: the stations are farther than %f degrees\n", opt.maxdist); return 0; }
  } else {
    opt.mindist = opt.maxdist = opt.VR = 0;
  }
  if (s1.Tr < o.mincc || t2.Tr < o.mincc) { printf("fpcc_fullpair: too few sequences\n"); return 0; }
  std::vector<int> i1 = select_traces(s1, o.stdn), i2 = o.acc ? i1 : select_traces(s2, o.stdn);
  if (o.autopair) {
    sort_by_time(s1, i1);
    if (o.acc) i2 = i1;
    else { sort_by_time(s2, i2); pair_lists(s1, i1, s2, i2); }
  } else {
    if (i1.size() != i2.size()) { printf("fpcc_fullpair: the lists have different lengths\n"); return -2; }
    for (size_t j = 0; j < i1.size(); j++)
      if (std::fabs(tdiff(s1.hdr[i1[j]], t2.hdr[i2[j]])) > 0.5) { printf("fpcc_fullpair: unpaired traces\n"); return 1; }
  }
  const int Tr = (int)i1.size();
  // lags
  int Lag1 = o.nl1 ? o.nl1 : (o.tl1 ? (int)std::lround(o.tl1 / (double)dt) : 0);
  int Lag2 = o.nl2 ? o.nl2 : (o.tl2 ? (int)std::lround(o.tl2 / (double)dt) : 0);
  if (Lag1 > Lag2) std::swap(Lag1, Lag2);
  if (std::abs(Lag1) >= N || std::abs(Lag2) >= N) { printf("fpcc_fullpair: TOO LARGE LAGS!!!\n"); return 6; }
  const int L = Lag2 - Lag1 + 1;
  printf("Lag1 = %d smpl (%d s), Lag2 = %d smpl (%d s), L = %d smpl (%d s), N = %d smpl, Tr = %d, gcarc = %f deg\n",
         Lag1, (int)(Lag1 * dt), Lag2, (int)(Lag2 * dt), L, (int)((L - 1) * dt), N, Tr, gcarc);
  if (Tr <= o.mincc) { printf("NO INTERSTATION CORRELATION TO BE COMPUTED.\n"); return 0; }
  std::vector<TraceHeader> h1(Tr), h2(Tr);
  for (int t = 0; t < Tr; t++) { h1[t] = s1.hdr[i1[t]]; h2[t] = t2.hdr[i2[t]]; }

  // device: station-1 rows [0, Tr), station-2 rows [Tr, 2 Tr), uploaded row by row
  fpcc_ctx* ctx = nullptr;
  GCHECK(fpcc_create(&ctx, 0));
  cudaStream_t st = (cudaStream_t)fpcc_get_stream(ctx);
  const int rows = o.acc ? Tr : 2 * Tr;
  float* d_x = nullptr;
  if (cudaMalloc(&d_x, (size_t)2 * Tr * N * sizeof(float)) != cudaSuccess) { printf("fpcc_fullpair: out of device memory\n"); return 4; }
  for (int t = 0; t < Tr; t++) {
    cudaMemcpyAsync(d_x + (size_t)t * N, s1.x + (size_t)i1[t] * N, (size_t)N * 4, cudaMemcpyHostToDevice, st);
    if (!o.acc)
      cudaMemcpyAsync(d_x + (size_t)(Tr + t) * N, s2.x + (size_t)i2[t] * N, (size_t)N * 4, cudaMemcpyHostToDevice, st);
  }
  // preprocessing on the device: clipping, whitening per station, reversed components
  if (o.clip) GCHECK(fpcc_clip_rows(ctx, d_x, N, rows, N));
  if (o.awhite[0] > 0 && o.awhite[1] > o.awhite[0]) {
    GCHECK(fpcc_whiten_rows(ctx, d_x, N, Tr, N, o.awhite[0], o.awhite[1], dt));
    if (!o.acc) GCHECK(fpcc_whiten_rows(ctx, d_x + (size_t)Tr * N, N, Tr, N, o.awhite[0], o.awhite[1], dt));
  }
  // reversed components (src/rotlib.c:14-34): a sign flip, applied after the
  // linear steps above (both commute with it)
  std::vector<float> neg(N);
  auto flip = [&](std::vector<TraceHeader>& h, int row0) -> int {
    for (int t = 0; t < Tr; t++) {
      bool f = false;
      if (h[t].cmpinc == 180) { f = true; h[t].cmpinc = 0; }
      else if (h[t].cmpinc == 90 && h[t].cmpaz < 315 && h[t].cmpaz > 135) {
        f = true;
        h[t].cmpaz -= 180;
        if (h[t].cmpaz < 0) h[t].cmpaz += 360;
      }
      if (f) {
        float* d = d_x + (size_t)(row0 + t) * N;
        if (cudaMemcpyAsync(neg.data(), d, (size_t)N * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
          return FPCC_ECUDA;
        for (float& v : neg) v = -v;
        if (cudaMemcpyAsync(d, neg.data(), (size_t)N * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
          return FPCC_ECUDA;
      }
    }
    return 0;
  };
  GCHECK(flip(h1, 0));
  if (!o.acc) GCHECK(flip(h2, Tr));
  if (o.acc) h2 = h1;
  const int row2 = o.acc ? 0 : Tr;

  std::vector<int32_t> pairs(2 * Tr);
  for (int t = 0; t < Tr; t++) { pairs[2 * t] = t; pairs[2 * t + 1] = row2 + t; }
  int32_t* d_pairs = nullptr;
  float* d_y = nullptr;
  cudaMalloc(&d_pairs, pairs.size() * 4);
  cudaMalloc(&d_y, (size_t)Tr * L * 4);
  cudaMemcpyAsync(d_pairs, pairs.data(), pairs.size() * 4, cudaMemcpyHostToDevice, st);
  std::vector<float> y((size_t)Tr * L);
  std::vector<std::thread> writers;
  // ts-PWS family in samples: pmin/pmax as given (seconds), else the WPCC defaults
  double spmin = 1.25 * std::sqrt(2.0) * 3.14159265358979323846, spmax = spmin * std::pow(2.0, 3.5);
  if (o.pmin != 0 && o.pmax != 0) { spmin = o.pmin / dt; spmax = o.pmax / dt; }
  // stacks of each channel pair's windows (the sets of the binary output), one SAC file per kind
  auto stack_sets = [&](const char* name) -> int {
    std::vector<char> done(Tr, 0);
    float *d_g = nullptr, *d_o = nullptr;
    if (cudaMalloc(&d_g, (size_t)Tr * L * 4) != cudaSuccess || cudaMalloc(&d_o, (size_t)L * 4) != cudaSuccess)
      return FPCC_ENOMEM;
    std::vector<float> ys(L);
    int rc = 0;
    for (int next = 0; next < Tr && !rc; next++) {
      if (done[next]) continue;
      std::vector<int> set;
      for (int t = next; t < Tr; t++)
        if (!done[t] && !strcmp(h1[t].chn, h1[next].chn) && !strcmp(h2[t].chn, h2[next].chn)) {
          done[t] = 1;
          set.push_back(t);
        }
      const int K = (int)set.size();
      bool contig = true;
      for (int i = 1; i < K; i++) contig &= set[i] == set[0] + i;
      const float* base = d_y + (size_t)set[0] * L;
      if (!contig) {
        for (int i = 0; i < K; i++)
          cudaMemcpyAsync(d_g + (size_t)i * L, d_y + (size_t)set[i] * L, (size_t)L * 4, cudaMemcpyDeviceToDevice, st);
        base = d_g;
      }
      static const char* kinds[3] = {"lin", "pws", "tspws"};
      for (int k = 0; k < 3 && !rc; k++) {
        if (!(o.stack & (1 << k))) continue;
        rc = fpcc_stack(ctx, k, base, (int64_t)K * L, L, K, L, 1, o.nu, spmin, spmax, (int)o.V, o.type, o.op1, d_o, L);
        if (rc) break;
        cudaMemcpyAsync(ys.data(), d_o, (size_t)L * 4, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        const TraceHeader &a = h1[set[0]], &b = h2[set[0]];
        char fn[200];
        snprintf(fn, sizeof fn, "%s.%s.%s.%s.%s.%s.%s.%s_%s_%s.sac", a.net, a.sta, a.loc, a.chn, b.net, b.sta, b.loc,
                 b.chn, name, kinds[k]);
        if (!write_sac(fn, ys.data(), L, Lag1 * dt, dt, name, a, b)) printf("fpcc_fullpair: error writing %s\n", fn);
      }
    }
    cudaFree(d_g);
    cudaFree(d_o);
    return rc;
  };
  int stack_rc = 0;
  auto emit = [&](const char* name) {
    cudaMemcpyAsync(y.data(), d_y, y.size() * 4, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (o.oformat == 1) store_sacs(y, L, Tr, Lag1, h1, h2, dt, name);
    else store_bins(y, L, Tr, Lag1, h1, h2, dt, name, o);
    if (o.stack && !stack_rc) stack_rc = stack_sets(name);
  };
  const int Nz = fpcc_choose_nz(N, Lag1, Lag2, FPCC_NZ_FAST);
  if (o.pcc) {
    const int m = (o.v == 2) ? FPCC_PCC2 : (o.v == 1 ? FPCC_PCC1 : FPCC_PCCV);
    const int64_t lds = m == FPCC_PCC2 ? Nz : N;
    void* d_s = nullptr;
    cudaMalloc(&d_s, (size_t)rows * lds * 8);
    GCHECK(fpcc_station_stage(ctx, m, d_x, N, rows, N, Nz, FPCC_F32, FPCC_AMP_F_REG, d_s, lds));
    GCHECK(fpcc_pair_stage(ctx, m, d_s, lds, FPCC_F32, d_pairs, Tr, N, Nz, Lag1, Lag2, (float)o.v, nullptr, 0,
                           d_y, L, nullptr));
    char nick[16];
    if (o.v == 2) strcpy(nick, "pcc2");
    else if (o.v == 1) strcpy(nick, "pcc1");
    else snprintf(nick, sizeof nick, "pcc%.1f", o.v);
    emit(nick);
    cudaFree(d_s);
  }
  if (o.wpcc) {
    double pmin = 1.25 * std::sqrt(2.0) * 3.14159265358979323846, pmax = pmin * std::pow(2.0, 3.5);
    if (o.pmin != 0 && o.pmax != 0) {
      pmin = o.pmin / dt;
      if (opt.VR == 0) pmax = o.pmax / dt;
      else pmax = std::min(111.19 * gcarc / (3 * opt.VR), o.pmax) / dt;
    }
    printf("pmin = %f smpl (%f s), pmax = %f smpl (%f s)\n", pmin, pmin * dt, pmax, pmax * dt);
    fpcc_wpcc_plan* p = nullptr;
    GCHECK(fpcc_wpcc_plan_create(ctx, &p, (unsigned)N, Lag1, Lag2, pmin, pmax, o.V, o.type, o.op1, FPCC_AMP_D_REG,
                                 FPCC_NZ_FAST));
    int wnz = 0, S = 0, wl = 0;
    fpcc_wpcc_plan_info(p, &wnz, &S, &wl);
    void* d_P = nullptr;
    if (cudaMalloc(&d_P, (size_t)rows * S * wnz * 8) != cudaSuccess) { printf("fpcc_fullpair: out of device memory\n"); return 4; }
    GCHECK(fpcc_wpcc_station_stage(ctx, p, d_x, N, rows, d_P, FPCC_F32));
    GCHECK(fpcc_wpcc_pair_stage(ctx, p, d_P, FPCC_F32, d_pairs, Tr, d_y, L));
    emit("wpcc2");
    cudaFree(d_P);
    fpcc_wpcc_plan_destroy(p);
  }
  if (o.ccgn) {
    const int H = Nz / 2 + 1;
    void* d_s = nullptr;
    double* d_E = nullptr;
    cudaMalloc(&d_s, (size_t)rows * H * 8);
    // energy rows with room for the normalisation tables: 2 (N + 1) doubles
    const int64_t ldE = 2 * ((int64_t)N + 1);
    cudaMalloc(&d_E, (size_t)rows * ldE * 8);
    GCHECK(fpcc_station_stage(ctx, FPCC_GNCC, d_x, N, rows, N, Nz, FPCC_F32, 0, d_s, H));
    GCHECK(fpcc_energy_stage(ctx, d_x, N, rows, N, d_E, ldE));
    GCHECK(fpcc_pair_stage(ctx, FPCC_GNCC, d_s, H, FPCC_F32, d_pairs, Tr, N, Nz, Lag1, Lag2, 0.f, d_E, ldE, d_y,
                           L, nullptr));
    emit("ccgn");
    cudaFree(d_s);
    cudaFree(d_E);
  }
  if (o.cc1b) {
    // the sign of an exact zero follows the trace's role (src/FFTapps.c:1037,1042):
    // station-1 rows x >= 0 -> +1, station-2 rows x > 0 -> +1 (separate rows also when auto-correlating)
    const int H = Nz / 2 + 1;
    void* d_s = nullptr;
    cudaMalloc(&d_s, (size_t)2 * Tr * H * 8);
    GCHECK(fpcc_station_stage(ctx, FPCC_CC1B, d_x, N, Tr, N, Nz, FPCC_F32, FPCC_SIGN_GE, d_s, H));
    GCHECK(fpcc_station_stage(ctx, FPCC_CC1B, d_x + (size_t)row2 * N, N, Tr, N, Nz, FPCC_F32, FPCC_SIGN_GT,
                              (char*)d_s + (size_t)Tr * H * 8, H));
    std::vector<int32_t> p1(2 * Tr);
    for (int t = 0; t < Tr; t++) { p1[2 * t] = t; p1[2 * t + 1] = Tr + t; }
    cudaMemcpyAsync(d_pairs, p1.data(), p1.size() * 4, cudaMemcpyHostToDevice, st);
    GCHECK(fpcc_pair_stage(ctx, FPCC_CC1B, d_s, H, FPCC_F32, d_pairs, Tr, N, Nz, Lag1, Lag2, 0.f, nullptr, 0, d_y,
                           L, nullptr));
    emit("cc1b");
    cudaFree(d_s);
  }
  if (stack_rc) {
    printf("fpcc_fullpair: stacking failed: %s\n", fpcc_last_error());
    return 4;
  }
  cudaFree(d_x);
  cudaFree(d_pairs);
  cudaFree(d_y);
  host_free(s1.x, s1.pinned);
  if (!o.acc) host_free(s2.x, s2.pinned);
  fpcc_destroy(ctx);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    puts("USAGE: fpcc_fullpair filelist1 filelist2 parameters (the parameters of PCC_fullpair_1b)");
    return 0;
  }
  Options o;
  if (parse(argc, argv, o)) return 1;
  return run(o);
}
