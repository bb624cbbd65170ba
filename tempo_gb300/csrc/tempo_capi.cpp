// tempo_capi.cpp -- the C ABI of libtempo_gb300 (declared in include/tempo_gb300.h).
//
// Host side of the drop-in: tempo_init (src/module_mp_tempo_driver.F90:42-182) builds a
// context that owns the device lookup tables; tempo_run (driver:187-513) validates
// the reference's argument list, sets up the column-step launch and, for host
// arrays, stages the tile through HBM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "tempo_gb300.h"
#include "tempo_internal.h"
#include "tempo_types.h"

using namespace tg;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
#define CUDA_TRY(expr)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(TEMPO_ERR_CUDA, "%s failed: %s", #expr, cudaGetErrorString(e_));      \
  } while (0)

template <class T>
int dev_alloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) return TEMPO_OK;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(TEMPO_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T),
                cudaGetErrorString(e));
  }
  return TEMPO_OK;
}

// host staging buffers reused across host-memory run calls
struct Mirror {
  void* d = nullptr;
  size_t bytes = 0;
};

}  // namespace

namespace {
constexpr size_t kGraphCache = 16;
// host-array runs: at most this many slabs of tile rows, each of at least about this
// many columns (the step kernels keep the GPU busy from about 2^17 columns up)
constexpr long kMaxSlabs = 8;
constexpr long kSlabColumns = 131072;
struct GraphEntry {
  std::string key;  // bytes of the step arguments + precision, variant, storage size
  cudaGraphExec_t exec;
};
}  // namespace

struct tempo_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  tempo_cfgs_t cfgs{};
  bool hail = true;
  int precision = TEMPO_PREC_FP64;
  TempoConsts<double> c64{};
  TempoConsts<float> c32{};
  IslandConsts<double> i64{};
  IslandConsts<df> idf{};
  TempoBins bins{};
  DevTables64 t64{};
  // FP32 copies for the mixed kernels
  float *f_efrw = nullptr, *f_efsw = nullptr, *f_tnc_wev = nullptr, *f_tps = nullptr,
        *f_tni = nullptr, *f_tpi = nullptr, *f_qg = nullptr, *f_qs = nullptr, *f_qrfz = nullptr,
        *f_qcfz = nullptr;
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  // second scratch and compute stream: host-array runs alternate slabs between the two
  // so that one slab's kernels overlap the next one's
  void* scratch2 = nullptr;
  size_t scratch2_bytes = 0;
  int scratch_slot = 0;
  cudaStream_t stream2 = nullptr;
  unsigned long long* d_stats = nullptr;
  long last_cols = 0;
  long launches = 0;
  std::vector<Mirror> mirrors;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool kernel_timing = false;
  cudaEvent_t kev[kStepPhases + 1] = {};
  int points_variant = 0;  // mixed form on FP32 storage (tempo_autotune_dev_f32_c)
  int points_order = 0;    // phase A's points level-major (0) or in regime order (1)
  int sedim_variant = 0;   // sedimentation kernel (tempo_set_sedim_variant)
  RadarConsts radar{};     // melting-layer reflectivity (FP64)
  double* d_mlnet = nullptr;  // cloud-number network (tempo_set_ml_cloud_number_c)
  bool use_graphs = false;
  std::vector<GraphEntry> graphs;  // captured steps, oldest first
  // host-array runs: copy streams and per-slab events of the pipelined copies, and
  // whether a run keeps the step counters of the slabs before it
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  std::vector<cudaEvent_t> slab_ev;
  bool keep_stats = false;
  int host_slabs = 0;  // slabs of a host-array run (0: from the tile's size)
  bool times_valid = false;  // the last run recorded the kernel-timing events
  bool validate = false;     // input scan before each run (tempo_set_validation)
  bool in_host_run = false;  // run_dev called by run_host (inputs scanned on the host)
  unsigned long long* d_first_bad = nullptr;  // result of the device input scan
#ifdef TEMPO_TRACE
  int* trace = nullptr;  // decision-trace buffer of a test build (tempo_set_trace_c)
#endif
};

namespace {

void free_tables(tempo_ctx* c) {
  double* d[] = {c->t64.t_efrw, c->t64.t_efsw, c->t64.tpc_wev, c->t64.tnc_wev, c->t64.tps_iaus,
                 c->t64.tni_iaus, c->t64.tpi_ide, c->t64.qg, c->t64.qs, c->t64.qrfz, c->t64.qcfz};
  for (double* p : d) cudaFree(p);
  cudaFree(c->t64.tnccn);
  cudaFree(c->t64.edges);
  float* f[] = {c->f_efrw, c->f_efsw, c->f_tnc_wev, c->f_tps, c->f_tni, c->f_tpi,
                c->f_qg,   c->f_qs,   c->f_qrfz,    c->f_qcfz};
  for (float* p : f) cudaFree(p);
  c->t64 = DevTables64{};
}

int alloc_tables(tempo_ctx* c) {
  int rc;
  DevTables64& t = c->t64;
  if ((rc = dev_alloc(&t.t_efrw, (size_t)nbr * nbc))) return rc;
  if ((rc = dev_alloc(&t.t_efsw, (size_t)nbs * nbc))) return rc;
  if ((rc = dev_alloc(&t.tpc_wev, (size_t)nbc * ntb_c * nbc))) return rc;
  if ((rc = dev_alloc(&t.tnc_wev, (size_t)nbc * ntb_c * nbc))) return rc;
  if ((rc = dev_alloc(&t.tps_iaus, (size_t)ntb_i * ntb_i1))) return rc;
  if ((rc = dev_alloc(&t.tni_iaus, (size_t)ntb_i * ntb_i1))) return rc;
  if ((rc = dev_alloc(&t.tpi_ide, (size_t)ntb_i * ntb_i1))) return rc;
  if ((rc = dev_alloc(&t.qg, (size_t)QG_COUNT * 5))) return rc;
  if ((rc = dev_alloc(&t.qs, (size_t)QS_COUNT * 12))) return rc;
  if ((rc = dev_alloc(&t.qrfz, (size_t)QRFZ_COUNT * 4))) return rc;
  if ((rc = dev_alloc(&t.qcfz, (size_t)QCFZ_COUNT * 2))) return rc;
  if ((rc = dev_alloc(&t.tnccn, (size_t)CCN_COUNT))) return rc;
  if ((rc = dev_alloc(&t.edges, (size_t)kEdgesCount))) return rc;
  return TEMPO_OK;
}

// the context's tables for the kernels of element type T (FP32 copies for float)
template <class T> Tables<T> tables_of(const tempo_ctx* c);
template <> Tables<double> tables_of<double>(const tempo_ctx* c) {
  return Tables<double>{c->t64.t_efrw, c->t64.t_efsw, c->t64.tnc_wev, c->t64.tps_iaus, c->t64.tni_iaus,
                        c->t64.tpi_ide, c->t64.tnccn, c->t64.qg, c->t64.qs, c->t64.qrfz, c->t64.qcfz,
                        c->t64.edges};
}
template <> Tables<float> tables_of<float>(const tempo_ctx* c) {
  return Tables<float>{c->f_efrw, c->f_efsw, c->f_tnc_wev, c->f_tps, c->f_tni, c->f_tpi,
                       c->t64.tnccn, c->f_qg, c->f_qs, c->f_qrfz, c->f_qcfz, c->t64.edges};
}

int make_f32_tables(tempo_ctx* c) {
  struct P {
    float** f;
    const double* d;
    long n;
  } ps[] = {{&c->f_efrw, c->t64.t_efrw, (long)nbr * nbc},
            {&c->f_efsw, c->t64.t_efsw, (long)nbs * nbc},
            {&c->f_tnc_wev, c->t64.tnc_wev, (long)nbc * ntb_c * nbc},
            {&c->f_tps, c->t64.tps_iaus, (long)ntb_i * ntb_i1},
            {&c->f_tni, c->t64.tni_iaus, (long)ntb_i * ntb_i1},
            {&c->f_tpi, c->t64.tpi_ide, (long)ntb_i * ntb_i1},
            {&c->f_qg, c->t64.qg, QG_COUNT * 5},
            {&c->f_qs, c->t64.qs, QS_COUNT * 12},
            {&c->f_qrfz, c->t64.qrfz, QRFZ_COUNT * 4},
            {&c->f_qcfz, c->t64.qcfz, QCFZ_COUNT * 2}};
  for (auto& p : ps) {
    if (!*p.f) {
      int rc = dev_alloc(p.f, (size_t)p.n);
      if (rc) return rc;
    }
    CUDA_TRY(narrow_copy(*p.f, p.d, p.n, c->stream));
  }
  return TEMPO_OK;
}

bool host_little() {
  uint16_t x = 1;
  return *(uint8_t*)&x == 1;
}
void bswap8(void* p, size_t n) {
  uint8_t* b = (uint8_t*)p;
  for (size_t i = 0; i < n; i++, b += 8)
    for (int k = 0; k < 4; k++) {
      uint8_t t = b[k];
      b[k] = b[7 - k];
      b[7 - k] = t;
    }
}

std::string join(const char* dir, const char* name) {
  std::string s = dir ? dir : ".";
  if (!s.empty() && s.back() != '/') s += '/';
  return s + name;
}

// ---- table files (driver:532-700) ---------------------------------------------------
// Largest value a collection or freezing table may hold: the tables are rates and
// probabilities far below it, while FP64 read in the wrong byte order gives values of
// any exponent.
constexpr double kTableMax = 1e30;

const char* table_file_of(const char* name) {
  if (!std::strcmp(name, "ccn_activate")) return "ccn_activate.bin";
  if (!std::strcmp(name, "qr_acr_qg")) return "qr_acr_qg_data_tempo_v3";
  if (!std::strcmp(name, "qr_acr_qs")) return "qr_acr_qs_data_tempo_v3";
  if (!std::strcmp(name, "freezewater")) return "freeze_water_data_tempo_v3";
  return nullptr;
}
// bytes of a table file: one Fortran record of FP32 for the CCN table, FP64 streams of
// the arrays in file order (tables.F90:122-127, 298-309, 438-442) for the others
long table_file_bytes(const char* name) {
  if (!std::strcmp(name, "ccn_activate")) return CCN_COUNT * 4 + 8;
  if (!std::strcmp(name, "qr_acr_qg")) return 5 * QG_COUNT * 8;
  if (!std::strcmp(name, "qr_acr_qs")) return 12 * QS_COUNT * 8;
  if (!std::strcmp(name, "freezewater")) return (4 * QRFZ_COUNT + 2 * QCFZ_COUNT) * 8;
  return -1;
}

// check_before_table_read (driver:652-700): the file exists and has the table's size
int check_table_size(const char* name, const char* path) {
  const long want = table_file_bytes(name);
  if (want < 0) return fail(TEMPO_ERR_ARG, "unknown table \"%s\" (ccn_activate, qr_acr_qg, qr_acr_qs, freezewater)", name);
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(TEMPO_ERR_TABLE, "table file \"%s\" was not found", path);
  std::fseek(f, 0, SEEK_END);
  const long size = std::ftell(f);
  std::fclose(f);
  if (size != want)
    return fail(TEMPO_ERR_TABLE, "table file \"%s\" has a size of %ld bytes but the %s table needs %ld bytes",
                path, size, name, want);
  return TEMPO_OK;
}

uint32_t be32(const uint8_t* b) {
  return (uint32_t)b[0] << 24 | (uint32_t)b[1] << 16 | (uint32_t)b[2] << 8 | (uint32_t)b[3];
}
double be64_double(const uint8_t* b) {
  uint64_t u = 0;
  for (int k = 0; k < 8; k++) u = u << 8 | b[k];
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}

// The content of the CCN file: record markers equal to the record's length, fractions
// in [0, 1].  buf holds the whole file.
int check_ccn_bytes(const std::vector<uint8_t>& buf, const char* path) {
  if (be32(buf.data()) != (uint32_t)(CCN_COUNT * 4) || std::memcmp(buf.data(), buf.data() + buf.size() - 4, 4))
    return fail(TEMPO_ERR_TABLE, "%s: bad record markers (expected %ld in big-endian order)", path,
                CCN_COUNT * 4);
  for (long i = 0; i < CCN_COUNT; i++) {
    const uint32_t u = be32(buf.data() + 4 + 4 * i);
    float v;
    std::memcpy(&v, &u, 4);
    if (!std::isfinite(v) || v < 0.f || v > 1.f)
      return fail(TEMPO_ERR_TABLE, "%s: activated fraction %g out of [0, 1] at %ld", path, (double)v, i);
  }
  return TEMPO_OK;
}

// one decoded value of a collection or freezing table
bool table_value_ok(double x) { return std::isfinite(x) && x >= 0.0 && x < kTableMax; }

// tempo_check_table_c: size, then every value
int check_table_file(const char* name, const char* path) {
  if (int rc = check_table_size(name, path)) return rc;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(TEMPO_ERR_TABLE, "cannot open %s", path);
  int rc = TEMPO_OK;
  if (!std::strcmp(name, "ccn_activate")) {
    std::vector<uint8_t> buf(CCN_COUNT * 4 + 8);
    if (std::fread(buf.data(), 1, buf.size(), f) != buf.size())
      rc = fail(TEMPO_ERR_TABLE, "%s: short read", path);
    else
      rc = check_ccn_bytes(buf, path);
  } else {
    const long n = table_file_bytes(name) / 8;
    std::vector<uint8_t> buf((size_t)1 << 23);
    for (long i0 = 0; i0 < n && rc == TEMPO_OK;) {
      const long m = std::min<long>(n - i0, (long)buf.size() / 8);
      if ((long)std::fread(buf.data(), 8, m, f) != m) {
        rc = fail(TEMPO_ERR_TABLE, "%s: short read", path);
        break;
      }
      for (long i = 0; i < m; i++) {
        const double x = be64_double(buf.data() + 8 * i);
        if (!table_value_ok(x)) {
          rc = fail(TEMPO_ERR_TABLE,
                    "%s: value %g at element %ld is negative, not finite or above %g (a file in "
                    "the wrong byte order reads so)", path, x, i0 + i, kTableMax);
          break;
        }
      }
      i0 += m;
    }
  }
  std::fclose(f);
  return rc;
}

// read_table_ccn (driver:625-649): Fortran sequential unformatted, big-endian FP32,
// one record of 8820 values between 4-byte length markers.
int read_ccn(tempo_ctx* c, const char* dir) {
  std::string path = join(dir, "ccn_activate.bin");
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(TEMPO_ERR_TABLE, "cannot open %s", path.c_str());
  std::vector<uint8_t> buf(CCN_COUNT * 4 + 8);
  size_t got = std::fread(buf.data(), 1, buf.size(), f);
  int extra = std::fgetc(f);
  std::fclose(f);
  if (got != buf.size() || extra != EOF)
    return fail(TEMPO_ERR_TABLE, "%s has the wrong size (expected %zu bytes)", path.c_str(), buf.size());
  if (int rc = check_ccn_bytes(buf, path.c_str())) return rc;
  std::vector<float> v(CCN_COUNT);
  for (long i = 0; i < CCN_COUNT; i++) {
    const uint32_t u = be32(buf.data() + 4 + 4 * i);
    std::memcpy(&v[i], &u, 4);
  }
  CUDA_TRY(cudaMemcpy(c->t64.tnccn, v.data(), CCN_COUNT * 4, cudaMemcpyHostToDevice));
  return TEMPO_OK;
}

// A big-endian FP64 stream table family: `narr` arrays of `counts[a]` doubles that
// land in AoS family `fam` (nfam wide) at slot `slot[a]`.
struct Family {
  const char* file;
  int narr;
  const long* counts;
  double** aos;  // per array: AoS destination base
  const int* nfam;
  const int* slot;
};

int read_stream_table(tempo_ctx* c, const std::string& path, int narr, const long* counts,
                      double* const* aos, const int* nfam, const int* slot) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(TEMPO_ERR_TABLE, "cannot open %s", path.c_str());
  long total = 0;
  for (int a = 0; a < narr; a++) total += counts[a];
  std::fseek(f, 0, SEEK_END);
  long size = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (size != total * 8) {
    std::fclose(f);
    return fail(TEMPO_ERR_TABLE, "%s has a size of %ld bytes but the table needs %ld bytes",
                path.c_str(), size, total * 8);
  }
  std::vector<double> host;
  double* dtmp = nullptr;
  long maxc = 0;
  for (int a = 0; a < narr; a++) maxc = counts[a] > maxc ? counts[a] : maxc;
  if (int rc = dev_alloc(&dtmp, (size_t)maxc)) {
    std::fclose(f);
    return rc;
  }
  for (int a = 0; a < narr; a++) {
    host.resize(counts[a]);
    if ((long)std::fread(host.data(), 8, counts[a], f) != counts[a]) {
      std::fclose(f);
      cudaFree(dtmp);
      return fail(TEMPO_ERR_TABLE, "%s: short read", path.c_str());
    }
    if (host_little()) bswap8(host.data(), counts[a]);
    for (long i = 0; i < counts[a]; i++)
      if (!table_value_ok(host[i])) {
        std::fclose(f);
        cudaFree(dtmp);
        return fail(TEMPO_ERR_TABLE,
                    "%s: array %d entry %ld = %g is negative, not finite or above %g (a file in the "
                    "wrong byte order reads so)", path.c_str(), a, i, host[i], kTableMax);
      }
    cudaError_t e = cudaMemcpy(dtmp, host.data(), counts[a] * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = aos_scatter(aos[a], dtmp, counts[a], nfam[a], slot[a], c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
      std::fclose(f);
      cudaFree(dtmp);
      return fail(TEMPO_ERR_CUDA, "table upload: %s", cudaGetErrorString(e));
    }
  }
  std::fclose(f);
  cudaFree(dtmp);
  return TEMPO_OK;
}

// reference file order of each family (tables.F90:122-127, 298-309, 438-442)
const long kFzCounts[6] = {QRFZ_COUNT, QRFZ_COUNT, QRFZ_COUNT, QRFZ_COUNT, QCFZ_COUNT, QCFZ_COUNT};
const int kFzNfam[6] = {4, 4, 4, 4, 2, 2};
const int kFzSlot[6] = {0, 1, 2, 3, 0, 1};  // tpi_qrfz tni_qrfz tpg_qrfz tnr_qrfz | tpi_qcfz tni_qcfz
const long kQsCounts[12] = {QS_COUNT, QS_COUNT, QS_COUNT, QS_COUNT, QS_COUNT, QS_COUNT,
                            QS_COUNT, QS_COUNT, QS_COUNT, QS_COUNT, QS_COUNT, QS_COUNT};
const int kQsNfam[12] = {12, 12, 12, 12, 12, 12, 12, 12, 12, 12, 12, 12};
const int kQsSlot[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
const long kQgCounts[5] = {QG_COUNT, QG_COUNT, QG_COUNT, QG_COUNT, QG_COUNT};
const int kQgNfam[5] = {5, 5, 5, 5, 5};
const int kQgSlot[5] = {0, 1, 2, 3, 4};

int read_big_tables(tempo_ctx* c, const char* dir) {
  double* fz[6] = {c->t64.qrfz, c->t64.qrfz, c->t64.qrfz, c->t64.qrfz, c->t64.qcfz, c->t64.qcfz};
  int rc = read_stream_table(c, join(dir, "freeze_water_data_tempo_v3"), 6, kFzCounts, fz, kFzNfam,
                             kFzSlot);
  if (rc) return rc;
  double* qs[12];
  for (int a = 0; a < 12; a++) qs[a] = c->t64.qs;
  rc = read_stream_table(c, join(dir, "qr_acr_qs_data_tempo_v3"), 12, kQsCounts, qs, kQsNfam, kQsSlot);
  if (rc) return rc;
  double* qg[5];
  for (int a = 0; a < 5; a++) qg[a] = c->t64.qg;
  return read_stream_table(c, join(dir, "qr_acr_qg_data_tempo_v3"), 5, kQgCounts, qg, kQgNfam, kQgSlot);
}

int build_tables_gpu(tempo_ctx* c, float* ms) {
  TempoConsts<double> hc;
  make_consts(&hc, true);  // tables are always built hail-aware (tables.F90:31,50)
  double* work = nullptr;
  if (int rc = dev_alloc(&work, big_tables_work_bytes() / sizeof(double))) return rc;
  CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
  cudaError_t e = build_big_tables(c->t64, c->bins, hc, work, big_tables_work_bytes(), c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(work);
  if (e != cudaSuccess) return fail(TEMPO_ERR_CUDA, "table build: %s", cudaGetErrorString(e));
  if (ms) cudaEventElapsedTime(ms, c->ev0, c->ev1);
  return TEMPO_OK;
}

// single_moment_nc_opt (cfgs:50-73): 'land' | 'ocean' | a number; typos fall back to land
double resolve_nc_value(const tempo_cfgs_t* cfg) {
  char buf[33];
  std::memcpy(buf, cfg->single_moment_nc_opt, 32);
  buf[32] = 0;
  char* s = buf;
  while (*s == ' ') s++;
  for (int i = (int)std::strlen(s) - 1; i >= 0 && (s[i] == ' ' || s[i] == 0); i--) s[i] = 0;
  if (!std::strcmp(s, "land")) return nt_c_l;
  if (!std::strcmp(s, "ocean")) return nt_c_o;
  char* end = nullptr;
  double v = std::strtod(s, &end);
  if (end == s) return nt_c_l;
  return v;
}

// the scratch of the context's current slot (c->scratch_slot), grown to `bytes`
int ensure_scratch(tempo_ctx* c, size_t bytes) {
  void*& scratch = c->scratch_slot ? c->scratch2 : c->scratch;
  size_t& have = c->scratch_slot ? c->scratch2_bytes : c->scratch_bytes;
  if (bytes <= have) return TEMPO_OK;
  cudaFree(scratch);
  scratch = nullptr;
  have = 0;
  cudaError_t e = cudaMalloc(&scratch, bytes);
  if (e != cudaSuccess)
    return fail(TEMPO_ERR_NOMEM, "scratch of %zu bytes: %s", bytes, cudaGetErrorString(e));
  have = bytes;
  return TEMPO_OK;
}

struct Bounds {
  int ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte;
};

int check_bounds(const Bounds& b) {
  if (b.ime < b.ims || b.jme < b.jms || b.kme < b.kms)
    return fail(TEMPO_ERR_ARG, "empty memory bounds");
  if (b.its < b.ims || b.ite > b.ime || b.jts < b.jms || b.jte > b.jme || b.kts < b.kms || b.kte > b.kme)
    return fail(TEMPO_ERR_ARG, "tile (%d:%d,%d:%d,%d:%d) outside memory (%d:%d,%d:%d,%d:%d)", b.its,
                b.ite, b.kts, b.kte, b.jts, b.jte, b.ims, b.ime, b.kms, b.kme, b.jms, b.jme);
  if (b.kte - b.kts + 1 < 2) return fail(TEMPO_ERR_ARG, "a column needs at least 2 levels");
  return TEMPO_OK;
}

template <class S>
struct RunArrays {
  S *t, *th;
  const S *pii, *p, *w, *dz;
  S *qv, *qc, *qr, *qi, *qs, *qg, *ni, *nr, *nc, *nwfa, *nifa, *ng, *qb;
  const int* land;
  const S *qc_bl = nullptr, *qcfrac_bl = nullptr;  // host path only
};

// Validates the argument list and launches the step on device arrays.
// Validates a run's arguments and fills the step arguments (everything but scratch).
// The checks of a run's arguments that need no context, in the order a caller reads
// them; run calls make them before they look at the context, so that a bad argument
// list is reported as such (TEMPO_ERR_ARG) whatever the context.
template <class S>
int check_run_args(const tempo_cfgs_t* cfg, double dt, const RunArrays<S>& A, const Bounds& b) {
  if (!cfg) return fail(TEMPO_ERR_ARG, "NULL tempo_cfgs");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(TEMPO_ERR_ARG, "dt must be > 0 (got %g)", dt);
  if (int rc = check_bounds(b)) return rc;
  if (!A.p || !A.w || !A.dz || !A.qv || !A.qc || !A.qr || !A.qi || !A.qs || !A.qg || !A.ni || !A.nr)
    return fail(TEMPO_ERR_ARG, "a required array (p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr) is NULL");
  if (!A.t && !(A.th && A.pii))
    return fail(TEMPO_ERR_ARG, "tempo_run requires either t or th and pii");
  return TEMPO_OK;
}

// the calling thread's current device must be the context's: the caller's stream and
// device arrays belong to it, and the context's tables live there
int check_current_device(const tempo_ctx* c) {
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return fail(TEMPO_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (cur != c->device)
    return fail(TEMPO_ERR_STATE,
                "the calling thread's current device is %d but the context lives on device %d "
                "(cudaSetDevice(%d) before a device-array call)", cur, c->device, c->device);
  return TEMPO_OK;
}

// The input fields of a run for the validation scan, with their names; t, th, pii, p
// and dz must be > 0, the others finite.
template <class S>
ValidateFields<S> validate_fields(const RunArrays<S>& A, const Bounds& b, const char** names) {
  ValidateFields<S> v{};
  const S* f[] = {A.t, A.th, A.pii, A.p, A.dz, A.w, A.qv, A.qc, A.qr, A.qi, A.qs, A.qg,
                  A.ni, A.nr, A.nc, A.nwfa, A.nifa, A.ng, A.qb};
  static const char* nm[] = {"t", "th", "pii", "p", "dz", "w", "qv", "qc", "qr", "qi", "qs",
                             "qg", "ni", "nr", "nc", "nwfa", "nifa", "ng", "qb"};
  const int n = (int)(sizeof f / sizeof f[0]);
  for (int i = 0; i < n; i++) {
    v.p[i] = f[i];
    v.positive[i] = i < 5;
    names[i] = nm[i];
  }
  v.nf = n;
  v.NI = (long)b.ime - b.ims + 1;
  v.NK = (long)b.kme - b.kms + 1;
  v.i0 = b.its - b.ims;
  v.k0 = b.kts - b.kms;
  v.j0 = b.jts - b.jms;
  v.ti = b.ite - b.its + 1;
  v.tj = b.jte - b.jts + 1;
  v.nz = b.kte - b.kts + 1;
  return v;
}

// the message of a failed scan: code = q * kValidateFields + f
template <class S>
int validation_failure(const ValidateFields<S>& v, const Bounds& b, const char** names,
                       unsigned long long code, double value) {
  const long q = (long)(code / kValidateFields);
  const int f = (int)(code % kValidateFields);
  const long i = q % v.ti, k = (q / v.ti) % v.nz, j = q / ((long)v.ti * v.nz);
  return fail(TEMPO_ERR_NONFINITE, "input %s(%ld, %ld, %ld) = %g is %s", names[f], b.its + i,
              b.kts + k, b.jts + j, value, v.positive[f] ? "not finite and > 0" : "not finite");
}

// The validation scan on host arrays, rows of the tile split over host threads.
template <class S>
int validate_host(const RunArrays<S>& A, const Bounds& b) {
  const char* names[kValidateFields];
  const ValidateFields<S> v = validate_fields(A, b, names);
  const int nthr = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<unsigned long long> first(nthr, ~0ull);
  std::vector<std::thread> pool;
  for (int t = 0; t < nthr; t++)
    pool.emplace_back([&, t] {
      for (long j = t; j < v.tj; j += nthr)
        for (long k = 0; k < v.nz; k++)
          for (long i = 0; i < v.ti; i++) {
            const long e = (v.i0 + i) + (v.k0 + k) * v.NI + (v.j0 + j) * v.NI * v.NK;
            const long q = i + v.ti * (k + (long)v.nz * j);
            for (int f = 0; f < v.nf; f++) {
              if (!v.p[f]) continue;
              const double x = (double)v.p[f][e];
              if (!std::isfinite(x) || (v.positive[f] && !(x > 0.0))) {
                first[t] = std::min(first[t], (unsigned long long)q * kValidateFields + f);
                break;
              }
            }
          }
    });
  for (auto& th : pool) th.join();
  const unsigned long long code = *std::min_element(first.begin(), first.end());
  if (code == ~0ull) return TEMPO_OK;
  const long q = (long)(code / kValidateFields);
  const long i = q % v.ti, k = (q / v.ti) % v.nz, j = q / ((long)v.ti * v.nz);
  const double x = (double)v.p[code % kValidateFields][(v.i0 + i) + (v.k0 + k) * v.NI + (v.j0 + j) * v.NI * v.NK];
  return validation_failure(v, b, names, code, x);
}

// The validation scan on device arrays: one kernel on stream s, then a wait for its result.
template <class S>
int validate_dev(tempo_ctx* c, const RunArrays<S>& A, const Bounds& b, cudaStream_t s) {
  const char* names[kValidateFields];
  const ValidateFields<S> v = validate_fields(A, b, names);
  unsigned long long code = ~0ull;
  CUDA_TRY(cudaMemcpyAsync(c->d_first_bad, &code, sizeof code, cudaMemcpyHostToDevice, s));
  CUDA_TRY(launch_validate(v, c->d_first_bad, s));
  CUDA_TRY(cudaMemcpyAsync(&code, c->d_first_bad, sizeof code, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (code == ~0ull) return TEMPO_OK;
  const long q = (long)(code / kValidateFields);
  const long i = q % v.ti, k = (q / v.ti) % v.nz, j = q / ((long)v.ti * v.nz);
  S x{};
  CUDA_TRY(cudaMemcpy(&x, v.p[code % kValidateFields] + (v.i0 + i) + (v.k0 + k) * v.NI + (v.j0 + j) * v.NI * v.NK,
                      sizeof x, cudaMemcpyDeviceToHost));
  return validation_failure(v, b, names, code, (double)x);
}

template <class S>
int build_args(tempo_ctx* c, const tempo_cfgs_t* cfg, double dt, int itimestep, const RunArrays<S>& A,
               const Bounds& b, const tempo_diags_t* dg, StepArgs<S>& a) {
  if (int rc = check_run_args(cfg, dt, A, b)) return rc;
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (A.qc_bl && A.qcfrac_bl && !c->d_mlnet)
    return fail(TEMPO_ERR_STATE, "the boundary-layer cloud path (qc_bl, qcfrac_bl) needs the "
                "cloud-number network (tempo_set_ml_cloud_number_c)");
  if (cfg->ml_for_nc_flag && !A.nc && !c->d_mlnet)
    return fail(TEMPO_ERR_STATE, "ml_for_nc_flag without nc needs the cloud-number network "
                "(tempo_set_ml_cloud_number_c)");
  uint32_t f = 0;
  if (A.nc) f |= F_NC;
  if (A.nwfa) f |= F_NWFA;
  if (A.nifa) f |= F_NIFA;
  if (A.ng && A.qb) f |= F_HAIL;
  if (A.qb) f |= F_QB;
  if (A.land) f |= F_LAND;
  if (itimestep == 1) f |= F_FIRST;
  if (cfg->turn_off_micro_flag) f |= F_NOMICRO;
  if (cfg->cloud_condensation_flag) f |= F_COND;
  if (cfg->refl10cm_flag) f |= F_REFL;
  if (cfg->re_cloud_flag && cfg->re_ice_flag && cfg->re_snow_flag) f |= F_RE;
  if (cfg->max_hail_diameter_flag) f |= F_MHD;
  if (cfg->rain_med_vol_diam_flag) f |= F_MVDR;
  if (cfg->graupel_med_vol_diam_flag) f |= F_MVDG;
  if (cfg->cloud_number_mixing_ratio_flag) f |= F_NCMR;
  if (A.t) f |= F_USE_T;
  if (dt > timestep_conversion_rime_to_rain) f |= F_DT_RIME;
  if (cfg->semi_sedi_flag) f |= F_SEMI;
  if (cfg->refl10cm_from_melting_flag && cfg->refl10cm_flag && dg && dg->refl10cm) f |= F_MELT;
  if (cfg->ml_for_nc_flag && !A.nc) f |= F_MLNC;
  if (A.qc_bl && A.qcfrac_bl) f |= F_BLRE;

  a = StepArgs<S>{};
  a.t = A.t;
  a.th = A.th;
  a.pii = A.pii;
  a.p = A.p;
  a.w = A.w;
  a.dz = A.dz;
  a.qv = A.qv;
  a.qc = A.qc;
  a.qr = A.qr;
  a.qi = A.qi;
  a.qs = A.qs;
  a.qg = A.qg;
  a.ni = A.ni;
  a.nr = A.nr;
  a.nc = A.nc;
  a.nwfa = A.nwfa;
  a.nifa = A.nifa;
  a.ng = A.ng;
  a.qb = A.qb;
  a.land = A.land;
  a.qc_bl = A.qc_bl;
  a.qcfrac_bl = A.qcfrac_bl;
  if (dg) {
    a.rain_precip = (S*)dg->rain_precip;
    a.ice_precip = (S*)dg->ice_liquid_equiv_precip;
    a.snow_precip = (S*)dg->snow_liquid_equiv_precip;
    a.graupel_precip = (S*)dg->graupel_liquid_equiv_precip;
    a.frozen_fraction = (S*)dg->frozen_fraction;
    a.frz_rain = (S*)dg->frz_rain_precip;
    if (cfg->max_hail_diameter_flag) {
      a.mhd_sfc = (S*)dg->max_hail_diameter_sfc;
      a.mhd_col = (S*)dg->max_hail_diameter_column;
    }
    if (cfg->refl10cm_flag) a.refl10cm = (S*)dg->refl10cm;
    if (cfg->re_cloud_flag) a.re_cloud = (S*)dg->re_cloud;
    if (cfg->re_ice_flag) a.re_ice = (S*)dg->re_ice;
    if (cfg->re_snow_flag) a.re_snow = (S*)dg->re_snow;
    if (cfg->rain_med_vol_diam_flag) a.mvd_r = (S*)dg->rain_med_vol_diam;
    if (cfg->graupel_med_vol_diam_flag) a.mvd_g = (S*)dg->graupel_med_vol_diam;
    if (cfg->cloud_number_mixing_ratio_flag) a.ncmr = (S*)dg->cloud_number_mixing_ratio;
  }
  a.NI = (long)b.ime - b.ims + 1;
  a.NK = (long)b.kme - b.kms + 1;
  a.i0 = b.its - b.ims;
  a.k0 = b.kts - b.kms;
  a.j0 = b.jts - b.jms;
  a.ti = b.ite - b.its + 1;
  a.tj = b.jte - b.jts + 1;
  a.nz = b.kte - b.kts + 1;
  a.ncol = (long)a.ti * a.tj;
  a.ncol_pad = (a.ncol + 31) / 32 * 32;
  a.dt = dt;
  a.odt = 1.0 / dt;
  a.dt_hi = (float)dt;
  a.dt_lo = (float)(dt - (double)a.dt_hi);
  a.odt_f = (float)a.odt;
  a.nc_single = resolve_nc_value(cfg);
  a.flags = f;
  a.mlnet = (f & (F_MLNC | F_BLRE)) ? c->d_mlnet : nullptr;
#ifdef TEMPO_TRACE
  a.trace = c->trace;
#endif
  // decay rates of the aerosol initial profiles (init_*_friendly_aerosols,
  // aerosols:14-73; h_01 = 0.8 km), host libm as in the reference
  a.niccn3 = -1.0 * std::log(naccn1 / naccn0) / 0.8;
  a.niin3 = -1.0 * std::log(nain1 / nain0) / 0.8;
  return TEMPO_OK;
}

template <class S>
int run_dev(tempo_ctx* c, const tempo_cfgs_t* cfg, double dt, int itimestep, const RunArrays<S>& A,
            const Bounds& b, const tempo_diags_t* dg, cudaStream_t s) {
  StepArgs<S> a;
  if (int rc = build_args(c, cfg, dt, itimestep, A, b, dg, a)) return rc;
  if (int rc = check_current_device(c)) return rc;
  if (c->validate && !c->in_host_run)
    if (int rc = validate_dev(c, A, b, s)) return rc;
  const bool mixed = c->precision == TEMPO_PREC_MIXED;
  // scratch: island-type point fields (double or double-float, 8 bytes either way),
  // bulk-type fall speeds, per-slot sums, slot map, masks and the slot counter
  const size_t rsz = mixed ? sizeof(float) : sizeof(double);
  const size_t npad = (size_t)a.ncol_pad, nzs = (size_t)a.nz;
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t sd_bytes = al((size_t)SD_N * nzs * npad * 8);
  const size_t sr_bytes = al((size_t)SR_N * nzs * npad * rsz);
  const size_t sc_bytes = al((size_t)SC_N * npad * 8);
  const size_t act_bytes = al(npad * sizeof(int));
  const size_t pm_bytes = al(nzs * npad);
  const size_t cm_bytes = al(npad);
  const size_t hg_bytes = al(nzs * npad * rsz);
  // semi-Lagrangian work rows (island type, 8 bytes) only on that path
  const size_t sl_bytes = (a.flags & F_SEMI) ? al((size_t)kSlRows * (nzs + 2) * npad * 8) : 0;
  // melting-reflectivity record of phase C only on that path
  const size_t ml_bytes = (a.flags & F_MELT) ? al((size_t)kMeltN * nzs * npad * 8 + nzs * npad) : 0;
  // per-point cloud number of the network only on that path
  const size_t nc_bytes = (a.flags & F_MLNC) ? al(nzs * npad * rsz) : 0;
  // regime order: a point index per point
  const bool order = c->points_order != 0;
  const size_t od_bytes = order ? al(nzs * npad * sizeof(unsigned)) : 0;
  const size_t total = sd_bytes + sr_bytes + sc_bytes + act_bytes + pm_bytes + cm_bytes + hg_bytes +
                       sl_bytes + ml_bytes + nc_bytes + od_bytes + 256;
  if (int rc = ensure_scratch(c, total)) return rc;
  char* sp = (char*)(c->scratch_slot ? c->scratch2 : c->scratch);
  a.sd = sp;
  sp += sd_bytes;
  a.sr = sp;
  sp += sr_bytes;
  a.sc = sp;
  sp += sc_bytes;
  a.act = (int*)sp;
  sp += act_bytes;
  a.pmask = (uint8_t*)sp;
  sp += pm_bytes;
  a.cmask = (uint8_t*)sp;
  sp += cm_bytes;
  a.hgt = sp;
  sp += hg_bytes;
  a.slw = sl_bytes ? sp : nullptr;
  sp += sl_bytes;
  a.mlw = ml_bytes ? sp : nullptr;
  sp += ml_bytes;
  a.ncw = nc_bytes ? sp : nullptr;
  sp += nc_bytes;
  a.ord = order ? (unsigned*)sp : nullptr;
  sp += od_bytes;
  a.nact = (unsigned int*)sp;
  a.stats = c->d_stats;
  c->last_cols = a.ncol;
  c->launches = kStepLaunches + (order ? kOrderLaunches : 0) + ((a.flags & F_MELT) ? 1 : 0);
  if (!mixed && sizeof(S) != sizeof(double))
    return fail(TEMPO_ERR_STATE, "FP32 arrays need TEMPO_PREC_MIXED (tempo_set_precision)");
  const bool timed = c->kernel_timing;
  c->times_valid = timed;
  // the step's work on stream st: counters reset, then the four kernels
  auto enqueue = [&](cudaStream_t st) -> cudaError_t {
    cudaError_t e = c->keep_stats ? cudaSuccess
                                  : cudaMemsetAsync(c->d_stats, 0, 8 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.nact, 0, 2 * sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    const cudaEvent_t* ev = timed ? c->kev : nullptr;
    if (!mixed) {
      if constexpr (sizeof(S) == sizeof(double)) {
        const Tables<double> T = tables_of<double>(c);
        e = launch_step_f64(a, T, c->c64, c->i64, st, ev, c->sedim_variant);
        return e == cudaSuccess ? launch_melt_refl(a, c->c64, c->radar, st) : e;
      }
      return cudaErrorInvalidValue;
    }
    const Tables<float> T = tables_of<float>(c);
    if constexpr (sizeof(S) == sizeof(double))
      e = launch_step_mixed_f64(a, T, c->c32, c->idf, st, ev, c->sedim_variant);
    else
      e = launch_step_mixed_f32(a, T, c->c32, c->idf, st, ev, c->points_variant, c->sedim_variant);
    // the melting-layer reflectivity pass (F_MELT) after phase C, outside the timed kernels
    return e == cudaSuccess ? launch_melt_refl(a, c->c64, c->radar, st) : e;
  };
  if (!c->use_graphs) {
    CUDA_TRY(enqueue(s));
    return TEMPO_OK;
  }
  // CUDA graph: captured once per distinct argument set, replayed on the caller's stream
  std::string key((const char*)&a, sizeof a);
  key.push_back((char)c->precision);
  key.push_back((char)c->points_variant);  // (the regime order changes a.ord)
  key.push_back((char)c->sedim_variant);
  key.push_back((char)c->keep_stats);
  key.push_back((char)sizeof(S));
  key.push_back((char)timed);  // event-record nodes around the kernels
  cudaGraphExec_t exec = nullptr;
  for (auto& g : c->graphs)
    if (g.key == key) exec = g.exec;
  if (!exec) {
    cudaGraph_t graph = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue(c->stream);
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return fail(TEMPO_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(TEMPO_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    if (c->graphs.size() >= kGraphCache) {
      cudaGraphExecDestroy(c->graphs.front().exec);
      c->graphs.erase(c->graphs.begin());
    }
    c->graphs.push_back(GraphEntry{key, exec});
  }
  CUDA_TRY(cudaGraphLaunch(exec, s));
  return TEMPO_OK;
}

// The mixed step on FP32 device arrays with its scratch in the fixed device array of
// tempo_noalloc.cu: no allocation, no graph, no timing events.  The scratch layout is
// run_dev's.
int run_dev_noalloc(tempo_ctx* c, const tempo_cfgs_t* cfg, double dt, int itimestep,
                    const RunArrays<float>& A, const Bounds& b, const tempo_diags_t* dg,
                    cudaStream_t s) {
  StepArgs<float> a;
  if (int rc = build_args(c, cfg, dt, itimestep, A, b, dg, a)) return rc;
  // the fixed scratch is looked up for c->device; kernels launched from another
  // current device would reach that device's array without peer access
  if (int rc = check_current_device(c)) return rc;
  if (a.flags & (F_SEMI | F_MELT | F_MLNC))
    return fail(TEMPO_ERR_UNSUPPORTED, "semi-Lagrangian sedimentation, the melting-layer reflectivity "
                "and the ML cloud number need work space beyond the fixed scratch of "
                "tempo_run_dev_f32_noalloc_c: call tempo_run_dev_f32_c");
  if (c->precision != TEMPO_PREC_MIXED)
    return fail(TEMPO_ERR_STATE, "FP32 arrays need TEMPO_PREC_MIXED (tempo_set_precision)");
  const size_t npad = (size_t)a.ncol_pad, nzs = (size_t)a.nz;
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t sd_bytes = al((size_t)SD_N * nzs * npad * 8);
  const size_t sr_bytes = al((size_t)SR_N * nzs * npad * sizeof(float));
  const size_t sc_bytes = al((size_t)SC_N * npad * 8);
  const size_t act_bytes = al(npad * sizeof(int));
  const size_t pm_bytes = al(nzs * npad);
  const size_t cm_bytes = al(npad);
  const size_t hg_bytes = al(nzs * npad * sizeof(float));
  const size_t total = sd_bytes + sr_bytes + sc_bytes + act_bytes + pm_bytes + cm_bytes + hg_bytes + 256;
  if (total > kNoAllocScratchBytes)
    return fail(TEMPO_ERR_ARG,
                "%ld columns x %d levels need %zu bytes of scratch; the fixed scratch of "
                "tempo_run_dev_f32_noalloc_c holds %zu (about %zu columns at this depth): "
                "split the tile or call tempo_run_dev_f32_c",
                a.ncol, a.nz, total, kNoAllocScratchBytes,
                kNoAllocScratchBytes / (total / std::max<size_t>(npad, 1)));
  void* base = nullptr;
  CUDA_TRY(noalloc_scratch(c->device, &base));
  char* sp = (char*)base;
  a.sd = sp;
  sp += sd_bytes;
  a.sr = sp;
  sp += sr_bytes;
  a.sc = sp;
  sp += sc_bytes;
  a.act = (int*)sp;
  sp += act_bytes;
  a.pmask = (uint8_t*)sp;
  sp += pm_bytes;
  a.cmask = (uint8_t*)sp;
  sp += cm_bytes;
  a.hgt = sp;
  sp += hg_bytes;
  a.nact = (unsigned int*)sp;
  a.stats = c->d_stats;
  c->last_cols = a.ncol;
  c->launches = kStepLaunches;
  c->times_valid = false;  // no timing events: an earlier run's times are not this step's
  if (c->validate)
    if (int rc = validate_dev(c, A, b, s)) return rc;
  // the slot counter and the statistics accumulate with atomics: zero them first;
  // every other scratch field is written before it is read
  CUDA_TRY(cudaMemsetAsync(c->d_stats, 0, 8 * sizeof(unsigned long long), s));
  CUDA_TRY(cudaMemsetAsync(a.nact, 0, 2 * sizeof(unsigned int), s));
  const Tables<float> T = tables_of<float>(c);
  CUDA_TRY(launch_step_mixed_f32(a, T, c->c32, c->idf, s, nullptr, c->points_variant, c->sedim_variant));
  return TEMPO_OK;
}

// The mixed step of a multi-domain batch on FP32 device arrays: each domain's arguments
// as run_dev builds them, scratch for every domain in the context's scratch, the batch's
// descriptors after them, one launch sequence (tempo_batch.cu).
int run_batch(tempo_ctx* c, const tempo_cfgs_t* cfg, int nd, const tempo_domain_t* doms, cudaStream_t s) {
  if (!doms || nd < 1 || nd > kMaxDomains)
    return fail(TEMPO_ERR_ARG, "ndomains must be in 1..%d with a domain array (got %d)", kMaxDomains, nd);
  if (!cfg) return fail(TEMPO_ERR_ARG, "NULL tempo_cfgs");
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (c->precision != TEMPO_PREC_MIXED)
    return fail(TEMPO_ERR_STATE, "the batch step runs the mixed form: tempo_set_precision(TEMPO_PREC_MIXED)");
  if (int rc = check_current_device(c)) return rc;
  std::vector<StepArgs<float>> A((size_t)nd);
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  struct Sizes {
    size_t sd, sr, sc, act, pm, cm, hg;
  };
  std::vector<Sizes> Z((size_t)nd);
  std::vector<long> col_start((size_t)nd + 1, 0);
  size_t total = 0;
  long npts_max = 0;
  for (int d = 0; d < nd; d++) {
    const tempo_domain_t& D = doms[d];
    const tempo_state_t& x = D.state;
    RunArrays<float> R{(float*)x.t, (float*)x.th, (const float*)x.pii, (const float*)x.p,
                       (const float*)x.w, (const float*)x.dz, (float*)x.qv, (float*)x.qc,
                       (float*)x.qr, (float*)x.qi, (float*)x.qs, (float*)x.qg, (float*)x.ni,
                       (float*)x.nr, (float*)x.nc, (float*)x.nwfa, (float*)x.nifa, (float*)x.ng,
                       (float*)x.qb, x.land_input};
    const Bounds b{D.ims, D.ime, D.jms, D.jme, D.kms, D.kme, D.its, D.ite, D.jts, D.jte, D.kts, D.kte};
    if (int rc = build_args(c, cfg, (double)D.dt, D.itimestep, R, b, &D.diags, A[d])) {
      const std::string why = g_err;
      return fail(rc, "domain %d: %s", d, why.c_str());
    }
    if (A[d].flags & (F_SEMI | F_MELT | F_MLNC | F_BLRE))
      return fail(TEMPO_ERR_UNSUPPORTED, "domain %d: the semi-Lagrangian, melting-layer and ML "
                  "cloud-number paths are not part of the batch step (tempo_run_dev_f32_c runs them)", d);
    const size_t npad = (size_t)A[d].ncol_pad, nzs = (size_t)A[d].nz;
    Sizes& z = Z[d];
    z.sd = al((size_t)SD_N * nzs * npad * 8);
    z.sr = al((size_t)SR_N * nzs * npad * sizeof(float));
    z.sc = al((size_t)SC_N * npad * 8);
    z.act = al(npad * sizeof(int));
    z.pm = al(nzs * npad);
    z.cm = al(npad);
    z.hg = al(nzs * npad * sizeof(float));
    total += z.sd + z.sr + z.sc + z.act + z.pm + z.cm + z.hg;
    col_start[d + 1] = col_start[d] + A[d].ncol;
    npts_max += A[d].ncol * A[d].nz;
  }
  if (npts_max >= (1L << 32))
    return fail(TEMPO_ERR_ARG, "a batch holds at most 2^32 - 1 column levels (got %ld)", npts_max);
  const bool order = c->points_order != 0;
  const size_t cnt_bytes = al((size_t)nd * 2 * sizeof(unsigned));   // each domain's counters
  const size_t dom_bytes = al((size_t)nd * sizeof(StepArgs<float>));
  const size_t cs_bytes = al(((size_t)nd + 1) * sizeof(long));
  const size_t plan_bytes = al((2 * ((size_t)nd + 1) + 1) * sizeof(unsigned));
  const size_t ord_bytes = order ? al((size_t)npts_max * sizeof(unsigned)) : 0;
  total += cnt_bytes + dom_bytes + cs_bytes + plan_bytes + ord_bytes + 256;
  if (int rc = ensure_scratch(c, total)) return rc;
  char* sp = (char*)c->scratch;
  unsigned* counters = (unsigned*)sp;
  sp += cnt_bytes;
  for (int d = 0; d < nd; d++) {
    StepArgs<float>& a = A[d];
    const Sizes& z = Z[d];
    a.sd = sp;
    sp += z.sd;
    a.sr = sp;
    sp += z.sr;
    a.sc = sp;
    sp += z.sc;
    a.act = (int*)sp;
    sp += z.act;
    a.pmask = (uint8_t*)sp;
    sp += z.pm;
    a.cmask = (uint8_t*)sp;
    sp += z.cm;
    a.hgt = sp;
    sp += z.hg;
    a.nact = counters + 2 * d;
    a.stats = c->d_stats;
    a.ord = nullptr;
  }
  StepArgs<float>* d_dom = (StepArgs<float>*)sp;
  sp += dom_bytes;
  long* d_cs = (long*)sp;
  sp += cs_bytes;
  unsigned* plan = (unsigned*)sp;
  sp += plan_bytes;
  unsigned* d_ord = order ? (unsigned*)sp : nullptr;
  BatchArgs<float> B{};
  B.dom = d_dom;
  B.col_start = d_cs;
  B.slot_start = plan;
  B.pt_start = plan + (nd + 1);
  B.queue = plan + 2 * (nd + 1);
  B.ord = d_ord;
  B.nd = nd;
  B.ncol = col_start[nd];
  B.npts_max = npts_max;
  c->last_cols = B.ncol;
  c->launches = kStepLaunches + 1 + (order ? kOrderLaunches : 0);
  const bool timed = c->kernel_timing;
  c->times_valid = timed;
  // descriptors from pageable host memory (staged before the call returns), counters zeroed
  CUDA_TRY(cudaMemcpyAsync(d_dom, A.data(), (size_t)nd * sizeof(StepArgs<float>), cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(d_cs, col_start.data(), ((size_t)nd + 1) * sizeof(long), cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemsetAsync(counters, 0, (size_t)nd * 2 * sizeof(unsigned), s));
  CUDA_TRY(cudaMemsetAsync(c->d_stats, 0, 8 * sizeof(unsigned long long), s));
  CUDA_TRY(launch_batch_mixed_f32(B, tables_of<float>(c), c->c32, c->idf, s, timed ? c->kev : nullptr,
                                  c->sedim_variant));
  return TEMPO_OK;
}

// Stages host arrays through device mirrors (whole memory extent), runs, copies back.
template <class S>
int run_host(tempo_ctx* c, const tempo_cfgs_t* cfg, double dt, int itimestep, const RunArrays<S>& H,
             const Bounds& b, tempo_diags_t* dg) {
  if (int rc = check_run_args(cfg, dt, H, b)) return rc;
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (c->validate)
    if (int rc = validate_host(H, b)) return rc;
  const size_t n3 = (size_t)(b.ime - b.ims + 1) * (b.kme - b.kms + 1) * (b.jme - b.jms + 1);
  const size_t n2 = (size_t)(b.ime - b.ims + 1) * (b.jme - b.jms + 1);
  const size_t t2 = (size_t)(b.ite - b.its + 1) * (b.jte - b.jts + 1);
  const size_t t3 = t2 * (b.kte - b.kts + 1);
  struct Slot {
    const void* h;
    size_t bytes;
    bool out;
  };
  const bool bl = H.qc_bl && H.qcfrac_bl;
  const S* in3[] = {H.t, H.th, H.pii, H.p, H.w, H.dz, H.qv, H.qc, H.qr, H.qi, H.qs, H.qg,
                    H.ni, H.nr, H.nc, H.nwfa, H.nifa, H.ng, H.qb,
                    bl ? H.qc_bl : nullptr, bl ? H.qcfrac_bl : nullptr};
  const bool out3[] = {true, true, false, false, false, false, true, true, true, true, true,
                       true, true, true, true, true, true, true, true, false, false};
  const int n_in = 21;
  void* dg_h[15] = {dg ? dg->rain_precip : nullptr, dg ? dg->ice_liquid_equiv_precip : nullptr,
                    dg ? dg->snow_liquid_equiv_precip : nullptr,
                    dg ? dg->graupel_liquid_equiv_precip : nullptr,
                    dg ? dg->frozen_fraction : nullptr, dg ? dg->frz_rain_precip : nullptr,
                    dg ? dg->max_hail_diameter_sfc : nullptr,
                    dg ? dg->max_hail_diameter_column : nullptr, dg ? dg->refl10cm : nullptr,
                    dg ? dg->re_cloud : nullptr, dg ? dg->re_ice : nullptr,
                    dg ? dg->re_snow : nullptr, dg ? dg->rain_med_vol_diam : nullptr,
                    dg ? dg->graupel_med_vol_diam : nullptr,
                    dg ? dg->cloud_number_mixing_ratio : nullptr};
  // diagnostics whose flag is off are not computed: the host arrays stay as they are
  // (no mirror, no copy back), as the reference leaves them unallocated (driver:302-386)
  const bool diag_on[15] = {true, true, true, true, true, true,
                            cfg && cfg->max_hail_diameter_flag, cfg && cfg->max_hail_diameter_flag,
                            cfg && cfg->refl10cm_flag, cfg && cfg->re_cloud_flag,
                            cfg && cfg->re_ice_flag, cfg && cfg->re_snow_flag,
                            cfg && cfg->rain_med_vol_diam_flag, cfg && cfg->graupel_med_vol_diam_flag,
                            cfg && cfg->cloud_number_mixing_ratio_flag};
  for (int i = 0; i < 15; i++)
    if (!diag_on[i]) dg_h[i] = nullptr;
  const int nslots = n_in + 1 + 15;
  if (c->mirrors.size() < (size_t)nslots) c->mirrors.resize(nslots);
  void* d[nslots];
  for (int i = 0; i < nslots; i++) {
    const void* h;
    size_t bytes;
    if (i < n_in) {
      h = in3[i];
      bytes = n3 * sizeof(S);
    } else if (i == n_in) {
      h = H.land;
      bytes = n2 * sizeof(int);
    } else {
      h = dg_h[i - n_in - 1];
      bytes = ((i - n_in - 1) < 8 ? t2 : t3) * sizeof(S);
    }
    d[i] = nullptr;
    if (!h) continue;
    Mirror& m = c->mirrors[i];
    if (m.bytes < bytes) {
      cudaFree(m.d);
      m.d = nullptr;
      m.bytes = 0;
      cudaError_t e = cudaMalloc(&m.d, bytes);
      if (e != cudaSuccess)
        return fail(TEMPO_ERR_NOMEM, "device mirror of %zu bytes: %s", bytes, cudaGetErrorString(e));
      m.bytes = bytes;
    }
    d[i] = m.d;
  }
  RunArrays<S> D{(S*)d[0],  (S*)d[1],  (const S*)d[2], (const S*)d[3], (const S*)d[4],
                 (const S*)d[5], (S*)d[6],  (S*)d[7],  (S*)d[8],  (S*)d[9],
                 (S*)d[10], (S*)d[11], (S*)d[12], (S*)d[13], (S*)d[14],
                 (S*)d[15], (S*)d[16], (S*)d[17], (S*)d[18], (const int*)d[n_in],
                 (const S*)d[19], (const S*)d[20]};
  // Slabs of tile rows j: the step is column-local and a slab of rows is one contiguous
  // range of every array (j is the slowest index), so slab i's copy to the device
  // (stream copy_in), its step and its copy back (copy_out) run beside the other slabs'
  // copies.  With two or more slabs (and no kernel timing) the steps alternate between
  // two compute streams, each with its own scratch, so that one slab's kernels overlap
  // the next one's.  Rows outside the tile are neither read nor written by the step
  // and are not copied.
  const long ti = b.ite - b.its + 1, nz = b.kte - b.kts + 1, nrows = b.jte - b.jts + 1;
  const long row3 = (long)(b.ime - b.ims + 1) * (b.kme - b.kms + 1), row2 = b.ime - b.ims + 1;
  const long want = c->host_slabs > 0 ? c->host_slabs : std::max<long>(1, (long)t2 / kSlabColumns);
  const int nslab = (int)std::min<long>(std::min<long>(kMaxSlabs, nrows), want);
  CUDA_TRY(cudaSetDevice(c->device));
  if (!c->copy_in) CUDA_TRY(cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking));
  if (!c->copy_out) CUDA_TRY(cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking));
  const bool two = nslab > 1 && !c->kernel_timing;
  if (two && !c->stream2) CUDA_TRY(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
  // the step counters start from zero before any slab (each slab then adds to them)
  CUDA_TRY(cudaMemsetAsync(c->d_stats, 0, 8 * sizeof(unsigned long long), c->copy_in));
  while (c->slab_ev.size() < (size_t)(2 * kMaxSlabs)) {
    cudaEvent_t e;
    CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c->slab_ev.push_back(e);
  }
  // slab weights: with four or more slabs the first and last are a quarter and the
  // second and second-to-last half of the others, so that the pipeline fills (the
  // first slab's copy in) and drains (the last slab's copy out) with little data
  long wsum = 0, wcum[kMaxSlabs + 1] = {0};
  for (int sl = 0; sl < nslab; sl++) {
    const int edge = std::min(sl, nslab - 1 - sl);
    wsum += (nslab >= 4) ? (edge == 0 ? 1 : edge == 1 ? 2 : 4) : 1;
    wcum[sl + 1] = wsum;
  }
  int rc = TEMPO_OK;
  long launches = 0;
  for (int sl = 0; sl < nslab && rc == TEMPO_OK; sl++) {
    const long ja = b.jts + (wcum[sl] * nrows) / wsum, jb = b.jts + (wcum[sl + 1] * nrows) / wsum - 1;
    if (jb < ja) continue;  // (only when a tile has fewer rows than the weights need)
    const long rows = jb - ja + 1;
    const size_t o3 = (size_t)(ja - b.jms) * row3, c3 = (size_t)rows * row3;
    const size_t o2 = (size_t)(ja - b.jms) * row2, c2 = (size_t)rows * row2;
    const size_t od2 = (size_t)(ja - b.jts) * ti, cd2 = (size_t)rows * ti;
    const size_t od3 = od2 * nz, cd3 = cd2 * nz;
    cudaEvent_t in_done = c->slab_ev[2 * sl], step_done = c->slab_ev[2 * sl + 1];
    for (int i = 0; i < n_in; i++)
      if (d[i])
        CUDA_TRY(cudaMemcpyAsync((S*)d[i] + o3, (const S*)in3[i] + o3, c3 * sizeof(S),
                                 cudaMemcpyHostToDevice, c->copy_in));
    if (d[n_in])
      CUDA_TRY(cudaMemcpyAsync((int*)d[n_in] + o2, H.land + o2, c2 * sizeof(int),
                               cudaMemcpyHostToDevice, c->copy_in));
    cudaStream_t cs = (two && (sl & 1)) ? c->stream2 : c->stream;
    CUDA_TRY(cudaEventRecord(in_done, c->copy_in));
    CUDA_TRY(cudaStreamWaitEvent(cs, in_done, 0));
    // the slab as a tile: rows ja..jb, diagnostics at the slab's offset in the tile
    Bounds bs = b;
    bs.jts = (int)ja;
    bs.jte = (int)jb;
    tempo_diags_t ddg{};
    void** ddp[15] = {&ddg.rain_precip, &ddg.ice_liquid_equiv_precip, &ddg.snow_liquid_equiv_precip,
                      &ddg.graupel_liquid_equiv_precip, &ddg.frozen_fraction, &ddg.frz_rain_precip,
                      &ddg.max_hail_diameter_sfc, &ddg.max_hail_diameter_column, &ddg.refl10cm,
                      &ddg.re_cloud, &ddg.re_ice, &ddg.re_snow, &ddg.rain_med_vol_diam,
                      &ddg.graupel_med_vol_diam, &ddg.cloud_number_mixing_ratio};
    for (int i = 0; i < 15; i++)
      *ddp[i] = d[n_in + 1 + i] ? (void*)((S*)d[n_in + 1 + i] + (i < 8 ? od2 : od3)) : nullptr;
    c->keep_stats = true;  // the counters sum (early exits) and take maxima over slabs
    c->in_host_run = true;
    c->scratch_slot = (two && (sl & 1)) ? 1 : 0;
    rc = run_dev(c, cfg, dt, itimestep, D, bs, &ddg, cs);
    c->keep_stats = false;
    c->in_host_run = false;
    c->scratch_slot = 0;
    if (rc) break;
    launches += c->launches;
    CUDA_TRY(cudaEventRecord(step_done, cs));
    CUDA_TRY(cudaStreamWaitEvent(c->copy_out, step_done, 0));
    for (int i = 0; i < n_in; i++)
      if (d[i] && out3[i])
        CUDA_TRY(cudaMemcpyAsync((S*)in3[i] + o3, (const S*)d[i] + o3, c3 * sizeof(S),
                                 cudaMemcpyDeviceToHost, c->copy_out));
    for (int i = 0; i < 15; i++)
      if (d[n_in + 1 + i]) {
        const size_t off = i < 8 ? od2 : od3, cnt = i < 8 ? cd2 : cd3;
        CUDA_TRY(cudaMemcpyAsync((S*)dg_h[i] + off, (const S*)d[n_in + 1 + i] + off, cnt * sizeof(S),
                                 cudaMemcpyDeviceToHost, c->copy_out));
      }
  }
  cudaError_t e1 = cudaStreamSynchronize(c->copy_in), e2 = cudaStreamSynchronize(c->stream),
              e3 = cudaStreamSynchronize(c->copy_out);
  if (c->stream2) {
    const cudaError_t e4 = cudaStreamSynchronize(c->stream2);
    if (e2 == cudaSuccess) e2 = e4;
  }
  if (rc) return rc;
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
    return fail(TEMPO_ERR_CUDA, "host-array run: %s",
                cudaGetErrorString(e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3));
  c->last_cols = (long)t2;
  c->launches = launches;
  return TEMPO_OK;
}

}  // namespace

extern "C" {

const char* tempo_version(void) { return "tempo_gb300 1.0 (TEMPO v3.1.1 column step, sm_103a)"; }
const char* tempo_last_error(void) { return g_err.c_str(); }

int tempo_default_cfgs(tempo_cfgs_t* c) {
  if (!c) return fail(TEMPO_ERR_ARG, "NULL cfgs");
  std::memset(c, 0, sizeof *c);
  c->aerosolaware_flag = 1;
  c->hailaware_flag = 1;
  c->cloud_condensation_flag = 1;
  std::strcpy(c->single_moment_nc_opt, "land");
  c->refl10cm_flag = 1;
  c->re_cloud_flag = 1;
  c->re_ice_flag = 1;
  c->re_snow_flag = 1;
  c->max_hail_diameter_flag = 1;
  return TEMPO_OK;
}

int tempo_init_c(const int* aerosolaware_flag, const int* hailaware_flag, const int* semi_sedi_flag,
                 const int* cloud_condensation_flag, const int* refl10cm_from_melting_flag,
                 const int* ml_for_bl_nc_flag, const int* ml_for_nc_flag, const int* force_init_flag,
                 tempo_cfgs_t* cfgs, const char* table_dir, int build_tables, int device,
                 tempo_ctx_t** out) {
  (void)force_init_flag;  // every context initialises its own tables
  if (!cfgs || !out) return fail(TEMPO_ERR_ARG, "tempo_cfgs and ctx must not be NULL");
  *out = nullptr;
  if (aerosolaware_flag) cfgs->aerosolaware_flag = *aerosolaware_flag != 0;
  if (hailaware_flag) cfgs->hailaware_flag = *hailaware_flag != 0;
  if (ml_for_bl_nc_flag) cfgs->ml_for_bl_nc_flag = *ml_for_bl_nc_flag != 0;
  if (ml_for_nc_flag) cfgs->ml_for_nc_flag = *ml_for_nc_flag != 0;
  if (semi_sedi_flag) cfgs->semi_sedi_flag = *semi_sedi_flag != 0;
  if (cloud_condensation_flag) cfgs->cloud_condensation_flag = *cloud_condensation_flag != 0;
  if (refl10cm_from_melting_flag) cfgs->refl10cm_from_melting_flag = *refl10cm_from_melting_flag != 0;

  // the table files first (existence and size, check_before_table_read, driver:652-700),
  // before any device work
  if (int rc = check_table_size("ccn_activate", join(table_dir, "ccn_activate.bin").c_str())) return rc;
  if (!build_tables)
    for (const char* nm : {"freezewater", "qr_acr_qs", "qr_acr_qg"})
      if (int rc = check_table_size(nm, join(table_dir, table_file_of(nm)).c_str())) return rc;
  if (device < 0) {
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return fail(TEMPO_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  }
  tempo_ctx* c = new (std::nothrow) tempo_ctx();
  if (!c) return fail(TEMPO_ERR_NOMEM, "context allocation failed");
  auto bail = [&](int rc) {
    tempo_ctx_destroy(c);
    return rc;
  };
  c->device = device;
  c->cfgs = *cfgs;
  c->hail = cfgs->hailaware_flag != 0;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return bail(fail(TEMPO_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e)));
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess)
    return bail(fail(TEMPO_ERR_CUDA, "stream/event creation: %s", cudaGetErrorString(e)));
  make_consts(&c->c64, c->hail);
  narrow_consts(c->c64, &c->c32);
  make_island_consts(c->c64, &c->i64);
  make_island_consts(c->c64, &c->idf);
  make_radar_consts(&c->radar);
  make_bins(&c->bins);
  int rc;
  if ((rc = alloc_tables(c))) return bail(rc);
  {
    double edges[kEdgesCount];
    make_index_edges(c->bins, edges);
    if ((e = cudaMemcpy(c->t64.edges, edges, sizeof edges, cudaMemcpyHostToDevice)) != cudaSuccess)
      return bail(fail(TEMPO_ERR_CUDA, "index edges: %s", cudaGetErrorString(e)));
  }
  if ((rc = dev_alloc(&c->d_stats, 8))) return bail(rc);
  if ((rc = dev_alloc(&c->d_first_bad, 1))) return bail(rc);
  e = build_small_tables(c->t64, c->bins, c->c64, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return bail(fail(TEMPO_ERR_CUDA, "small tables: %s", cudaGetErrorString(e)));
  if ((rc = read_ccn(c, table_dir))) return bail(rc);
  if (build_tables) {
    if ((rc = build_tables_gpu(c, nullptr))) return bail(rc);
  } else {
    if ((rc = read_big_tables(c, table_dir))) return bail(rc);
  }
  if ((rc = make_f32_tables(c))) return bail(rc);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return bail(fail(TEMPO_ERR_CUDA, "init: %s", cudaGetErrorString(e)));
  *out = c;
  return TEMPO_OK;
}

int tempo_ctx_destroy(tempo_ctx_t* c) {
  if (!c) return TEMPO_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_tables(c);
  cudaFree(c->scratch);
  cudaFree(c->scratch2);
  cudaFree(c->d_stats);
  cudaFree(c->d_first_bad);
  cudaFree(c->d_mlnet);
  for (auto& m : c->mirrors) cudaFree(m.d);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (cudaEvent_t& e : c->kev)
    if (e) cudaEventDestroy(e);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  for (cudaEvent_t e : c->slab_ev) cudaEventDestroy(e);
  if (c->copy_in) cudaStreamDestroy(c->copy_in);
  if (c->copy_out) cudaStreamDestroy(c->copy_out);
  if (c->stream2) cudaStreamSynchronize(c->stream2), cudaStreamDestroy(c->stream2);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return TEMPO_OK;
}

int tempo_set_precision(tempo_ctx_t* c, int precision) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (precision != TEMPO_PREC_FP64 && precision != TEMPO_PREC_MIXED)
    return fail(TEMPO_ERR_ARG, "unknown precision %d", precision);
  c->precision = precision;
  return TEMPO_OK;
}

#ifdef TEMPO_TRACE
// Test builds only (not part of the ABI): later runs record every table index and
// branch decision into the zeroed device buffer (TraceSlot layout, tempo_types.h),
// kTracePoint ints per (tile column, level) point and kTraceColumn per tile column; one
// tile per run (device-array runs, or host-array runs of one slab).  NULL: off.
int tempo_set_trace_c(tempo_ctx_t* c, void* dev_buffer) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  c->trace = (int*)dev_buffer;
  return TEMPO_OK;
}
#endif

int tempo_set_validation(tempo_ctx_t* c, int on) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  c->validate = on != 0;
  return TEMPO_OK;
}

int tempo_check_table_c(const char* name, const char* path) {
  if (!name || !path) return fail(TEMPO_ERR_ARG, "NULL name or path");
  return check_table_file(name, path);
}

int tempo_set_kernel_timing(tempo_ctx_t* c, int on) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  CUDA_TRY(cudaSetDevice(c->device));
  if (on && !c->kev[0])
    for (cudaEvent_t& e : c->kev) CUDA_TRY(cudaEventCreate(&e));
  c->kernel_timing = on != 0;
  return TEMPO_OK;
}

int tempo_kernel_times_c(tempo_ctx_t* c, float ms[5]) {
  if (!c || !ms) return fail(TEMPO_ERR_ARG, "NULL argument");
  if (!c->kernel_timing) return fail(TEMPO_ERR_STATE, "kernel timing is off (tempo_set_kernel_timing)");
  if (!c->times_valid)
    return fail(TEMPO_ERR_STATE, "the last run recorded no kernel times (no timed run yet, or "
                "tempo_run_dev_f32_noalloc_c, which records none)");
  CUDA_TRY(cudaSetDevice(c->device));
  CUDA_TRY(cudaEventSynchronize(c->kev[kStepPhases]));
  for (int i = 0; i < kStepPhases; i++) CUDA_TRY(cudaEventElapsedTime(&ms[i], c->kev[i], c->kev[i + 1]));
  return TEMPO_OK;
}

int tempo_run_c(tempo_ctx_t* c, const tempo_cfgs_t* cfg, double dt, int itimestep, double* t,
                double* th, const double* pii, const double* p, const double* w, const double* dz,
                double* qv, double* qc, double* qr, double* qi, double* qs, double* qg, double* ni,
                double* nr, double* nc, double* nwfa, double* nifa, double* ng, double* qb,
                const double* qc_bl, const double* qcfrac_bl, double* qcfrac, double* qifrac,
                const double* thten_bl, const double* qvten_bl, const double* qcten_bl,
                const double* qiten_bl, const double* thten_lwrad, const double* thten_swrad,
                const int* land_input, int ids, int ide, int jds, int jde, int kds, int kde, int ims,
                int ime, int jms, int jme, int kms, int kme, int its, int ite, int jts, int jte,
                int kts, int kte, tempo_diags_t* diags) {
  (void)qcfrac; (void)qifrac; (void)thten_bl; (void)qvten_bl; (void)qcten_bl; (void)qiten_bl;
  (void)thten_lwrad; (void)thten_swrad; (void)ids; (void)ide; (void)jds; (void)jde; (void)kds; (void)kde;
  if (c && c->precision != TEMPO_PREC_FP64 && c->precision != TEMPO_PREC_MIXED)
    return fail(TEMPO_ERR_STATE, "bad precision");
  RunArrays<double> H{t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb, land_input};
  H.qc_bl = qc_bl;  // with qcfrac_bl: the boundary-layer cloud in re_cloud (main:832-857)
  H.qcfrac_bl = qcfrac_bl;
  return run_host(c, cfg, dt, itimestep, H, Bounds{ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte}, diags);
}

int tempo_run_f32_c(tempo_ctx_t* c, const tempo_cfgs_t* cfg, float dt, int itimestep, float* t,
                    float* th, const float* pii, const float* p, const float* w, const float* dz,
                    float* qv, float* qc, float* qr, float* qi, float* qs, float* qg, float* ni,
                    float* nr, float* nc, float* nwfa, float* nifa, float* ng, float* qb,
                    const float* qc_bl, const float* qcfrac_bl, float* qcfrac, float* qifrac,
                    const float* thten_bl, const float* qvten_bl, const float* qcten_bl,
                    const float* qiten_bl, const float* thten_lwrad, const float* thten_swrad,
                    const int* land_input, int ids, int ide, int jds, int jde, int kds, int kde,
                    int ims, int ime, int jms, int jme, int kms, int kme, int its, int ite,
                    int jts, int jte, int kts, int kte, tempo_diags_t* diags) {
  (void)qcfrac; (void)qifrac; (void)thten_bl; (void)qvten_bl; (void)qcten_bl; (void)qiten_bl;
  (void)thten_lwrad; (void)thten_swrad; (void)ids; (void)ide; (void)jds; (void)jde; (void)kds; (void)kde;
  RunArrays<float> H{t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb, land_input};
  H.qc_bl = qc_bl;
  H.qcfrac_bl = qcfrac_bl;
  return run_host(c, cfg, (double)dt, itimestep, H, Bounds{ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte}, diags);
}

int tempo_run_dev_c(tempo_ctx_t* c, const tempo_cfgs_t* cfg, double dt, int itimestep, double* t,
                    double* th, const double* pii, const double* p, const double* w,
                    const double* dz, double* qv, double* qc, double* qr, double* qi, double* qs,
                    double* qg, double* ni, double* nr, double* nc, double* nwfa, double* nifa,
                    double* ng, double* qb, const int* land_input, int ims, int ime, int jms,
                    int jme, int kms, int kme, int its, int ite, int jts, int jte, int kts, int kte,
                    tempo_diags_t* diags, void* stream) {
  RunArrays<double> A{t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb, land_input};
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the default stream
  return run_dev(c, cfg, dt, itimestep, A, Bounds{ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte}, diags, s);
}

int tempo_run_dev_f32_c(tempo_ctx_t* c, const tempo_cfgs_t* cfg, float dt, int itimestep, float* t,
                        float* th, const float* pii, const float* p, const float* w,
                        const float* dz, float* qv, float* qc, float* qr, float* qi, float* qs,
                        float* qg, float* ni, float* nr, float* nc, float* nwfa, float* nifa,
                        float* ng, float* qb, const int* land_input, int ims, int ime, int jms,
                        int jme, int kms, int kme, int its, int ite, int jts, int jte, int kts,
                        int kte, tempo_diags_t* diags, void* stream) {
  RunArrays<float> A{t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb, land_input};
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the default stream
  return run_dev(c, cfg, (double)dt, itimestep, A, Bounds{ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte}, diags, s);
}

int tempo_run_dev_f32_noalloc_c(tempo_ctx_t* c, const tempo_cfgs_t* cfg, float dt, int itimestep,
                                float* t, float* th, const float* pii, const float* p,
                                const float* w, const float* dz, float* qv, float* qc, float* qr,
                                float* qi, float* qs, float* qg, float* ni, float* nr, float* nc,
                                float* nwfa, float* nifa, float* ng, float* qb,
                                const int* land_input, int ims, int ime, int jms, int jme, int kms,
                                int kme, int its, int ite, int jts, int jte, int kts, int kte,
                                tempo_diags_t* diags, void* stream) {
  RunArrays<float> A{t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb, land_input};
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the default stream
  return run_dev_noalloc(c, cfg, (double)dt, itimestep, A,
                         Bounds{ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte}, diags, s);
}

int tempo_autotune_dev_f32_c(tempo_ctx_t* c, const tempo_cfgs_t* cfg, float dt, int itimestep,
                             float* t, float* th, const float* pii, const float* p, const float* w,
                             const float* dz, float* qv, float* qc, float* qr, float* qi,
                             float* qs, float* qg, float* ni, float* nr, float* nc, float* nwfa,
                             float* nifa, float* ng, float* qb, const int* land_input, int ims,
                             int ime, int jms, int jme, int kms, int kme, int its, int ite, int jts,
                             int jte, int kts, int kte, tempo_diags_t* diags, void* stream,
                             int reps, float* times_ms, int count, int* chosen) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (c->precision != TEMPO_PREC_MIXED)
    return fail(TEMPO_ERR_STATE, "autotune needs TEMPO_PREC_MIXED (tempo_set_precision)");
  const Bounds b{ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte};
  if (int rc = check_bounds(b)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  CUDA_TRY(cudaSetDevice(c->device));
  if (reps < 1) reps = 1;
  // private copies of every array the step writes: the caller's state is untouched
  const size_t ext = (size_t)(ime - ims + 1) * (kme - kms + 1) * (jme - jms + 1);
  const size_t n2 = (size_t)(ite - its + 1) * (jte - jts + 1), n3 = n2 * (kte - kts + 1);
  float* io[] = {t, th, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb};
  constexpr int NIO = sizeof(io) / sizeof(io[0]);
  float* cp[NIO] = {};
  void** dsrc = diags ? (void**)diags : nullptr;
  constexpr int ND = sizeof(tempo_diags_t) / sizeof(void*);
  tempo_diags_t dcopy{};
  void** dd = (void**)&dcopy;
  auto release = [&]() {
    for (float* q : cp) cudaFree(q);
    for (int i = 0; i < ND; i++) cudaFree(dd[i]);
  };
  for (int i = 0; i < NIO; i++)
    if (io[i] && cudaMalloc(&cp[i], ext * sizeof(float)) != cudaSuccess) {
      release();
      return fail(TEMPO_ERR_NOMEM, "autotune: copy of the state (%zu floats)", ext);
    }
  for (int i = 0; i < ND; i++)
    if (dsrc && dsrc[i] && cudaMalloc(&dd[i], (i < 8 ? n2 : n3) * sizeof(float)) != cudaSuccess) {
      release();
      return fail(TEMPO_ERR_NOMEM, "autotune: diagnostic buffers");
    }
  const bool timing = c->kernel_timing;
  const int saved_variant = c->points_variant, saved_order = c->points_order,
            saved_sedim = c->sedim_variant;
  int rc = tempo_set_kernel_timing(c, 1);
  float best = 0.0f, best_sed = 0.0f;
  int best_v = saved_order * kPointsVariants + saved_variant, best_s = saved_sedim;
  // every candidate runs the same `reps` consecutive steps from a fresh copy of the
  // state (the work of a step depends on the state it starts from) and is scored by
  // the median of its per-step times (single steps of a workload can cost far more
  // than the others, and by amounts that vary from run to run).  Candidates
  // [0, kPointsCandidates): points variant v % kPointsVariants in point order
  // v / kPointsVariants, scored by the regime kernel and the points kernel; then the
  // sedimentation variants with the points candidate kept, scored by that kernel.
  std::vector<float> per_step((size_t)reps);
  for (int v = 0; v < kPointsCandidates + kSedimCandidates && rc == TEMPO_OK; v++) {
    const bool sed = v >= kPointsCandidates;
    const int pv = sed ? best_v : v;
    c->points_variant = pv % kPointsVariants;
    c->points_order = pv / kPointsVariants;
    c->sedim_variant = sed ? v - kPointsCandidates : saved_sedim;
    float vbest = 0.0f;
    for (int i = 0; i < NIO; i++)
      if (io[i] && cudaMemcpyAsync(cp[i], io[i], ext * sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        rc = fail(TEMPO_ERR_CUDA, "autotune: state copy");
    for (int r = 0; r < reps && rc == TEMPO_OK; r++) {
      RunArrays<float> A{cp[0], cp[1], pii, p, w, dz, cp[2], cp[3], cp[4], cp[5], cp[6],
                         cp[7], cp[8], cp[9], cp[10], cp[11], cp[12], cp[13], cp[14], land_input};
      rc = run_dev(c, cfg, (double)dt, itimestep + r, A, b, diags ? &dcopy : nullptr, s);
      float ms[kStepPhases];
      if (rc == TEMPO_OK) rc = tempo_kernel_times_c(c, ms);
      if (rc == TEMPO_OK) per_step[(size_t)r] = sed ? ms[3] : ms[1] + ms[2];
    }
    if (rc == TEMPO_OK) {
      std::sort(per_step.begin(), per_step.end());
      vbest = (reps % 2) ? per_step[(size_t)reps / 2]
                         : 0.5f * (per_step[(size_t)reps / 2 - 1] + per_step[(size_t)reps / 2]);
    }
    if (rc) break;
    if (times_ms && v < count) times_ms[v] = vbest;
    if (!sed && (v == 0 || vbest < best)) {
      best = vbest;
      best_v = v;
    }
    if (sed && (v == kPointsCandidates || vbest < best_sed)) {
      best_sed = vbest;
      best_s = v - kPointsCandidates;
    }
  }
  if (!timing) tempo_set_kernel_timing(c, 0);
  cudaStreamSynchronize(s);
  release();
  if (rc) {
    c->points_variant = saved_variant;
    c->points_order = saved_order;
    c->sedim_variant = saved_sedim;
    return rc;
  }
  c->points_variant = best_v % kPointsVariants;
  c->points_order = best_v / kPointsVariants;
  c->sedim_variant = best_s;
  if (chosen) *chosen = best_v;
  return TEMPO_OK;
}

int tempo_set_host_slabs(tempo_ctx_t* c, int slabs) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (slabs < 0 || slabs > kMaxSlabs) return fail(TEMPO_ERR_ARG, "slabs %d outside [0, %ld]", slabs, kMaxSlabs);
  c->host_slabs = slabs;
  return TEMPO_OK;
}

int tempo_tuning_c(tempo_ctx_t* c, int out[3]) {
  if (!c || !out) return fail(TEMPO_ERR_ARG, "NULL argument");
  out[0] = c->points_variant;
  out[1] = c->points_order;
  out[2] = c->sedim_variant;
  return TEMPO_OK;
}

int tempo_set_sedim_variant(tempo_ctx_t* c, int variant) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (variant < 0 || variant >= kSedimCandidates)
    return fail(TEMPO_ERR_ARG, "sedimentation variant %d outside [0, %d)", variant, kSedimCandidates);
  c->sedim_variant = variant;
  return TEMPO_OK;
}

int tempo_set_graphs(tempo_ctx_t* c, int on) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  c->use_graphs = on != 0;
  return TEMPO_OK;
}

int tempo_set_ml_cloud_number_c(tempo_ctx_t* c, const double* mean, const double* var,
                                const double* weights00, const double* bias00,
                                const double* weights01, const double* bias01) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (!mean || !var || !weights00 || !bias00 || !weights01 || !bias01)
    return fail(TEMPO_ERR_ARG, "a network array is NULL");
  double h[kMlNet];
  std::memcpy(h, mean, 7 * sizeof(double));
  std::memcpy(h + 7, var, 7 * sizeof(double));
  std::memcpy(h + 14, weights00, 168 * sizeof(double));
  std::memcpy(h + 182, bias00, 24 * sizeof(double));
  std::memcpy(h + 206, weights01, 24 * sizeof(double));
  h[230] = bias01[0];
  for (int i = 7; i < 14; i++)
    if (!(h[i] > 0.0)) return fail(TEMPO_ERR_ARG, "scaler variance %d is not positive", i - 7);
  CUDA_TRY(cudaSetDevice(c->device));
  if (!c->d_mlnet) {
    cudaError_t e = cudaMalloc(&c->d_mlnet, sizeof h);
    if (e != cudaSuccess) {
      c->d_mlnet = nullptr;
      return fail(TEMPO_ERR_NOMEM, "network weights: %s", cudaGetErrorString(e));
    }
  }
  CUDA_TRY(cudaMemcpy(c->d_mlnet, h, sizeof h, cudaMemcpyHostToDevice));
  return TEMPO_OK;
}

int tempo_set_points_variant(tempo_ctx_t* c, int variant) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (variant < 0 || variant >= kPointsVariants) return fail(TEMPO_ERR_ARG, "variant %d outside [0, %d)", variant, kPointsVariants);
  c->points_variant = variant;
  return TEMPO_OK;
}

int tempo_set_points_order(tempo_ctx_t* c, int order) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (order != 0 && order != 1) return fail(TEMPO_ERR_ARG, "point order %d is neither 0 nor 1", order);
  c->points_order = order;
  return TEMPO_OK;
}

}  // extern "C"

namespace {

// device buffers released when the scope ends (after a stream synchronisation)
struct DevBufs {
  std::vector<void*> p;
  ~DevBufs() {
    for (void* q : p) cudaFree(q);
  }
  template <class X>
  X* alloc(size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, (n ? n : 1) * sizeof(X)) != cudaSuccess) return nullptr;
    p.push_back(q);
    return (X*)q;
  }
};

template <class T>
RunArrays<T> arrays_of(const tempo_state_t* x) {
  return RunArrays<T>{(T*)x->t,  (T*)x->th, (const T*)x->pii, (const T*)x->p, (const T*)x->w,
                      (const T*)x->dz, (T*)x->qv, (T*)x->qc, (T*)x->qr, (T*)x->qi, (T*)x->qs,
                      (T*)x->qg, (T*)x->ni, (T*)x->nr, (T*)x->nc, (T*)x->nwfa, (T*)x->nifa,
                      (T*)x->ng, (T*)x->qb, x->land_input};
}

// scalar fields of the step arguments (all but pointers)
template <class A, class B>
void copy_scalars(A& d, const B& s) {
  d.NI = s.NI; d.NK = s.NK; d.i0 = s.i0; d.k0 = s.k0; d.j0 = s.j0; d.ti = s.ti; d.tj = s.tj;
  d.nz = s.nz; d.ncol = s.ncol; d.ncol_pad = s.ncol_pad; d.dt = s.dt; d.odt = s.odt;
  d.dt_hi = s.dt_hi; d.dt_lo = s.dt_lo; d.odt_f = s.odt_f; d.nc_single = s.nc_single;
  d.niccn3 = s.niccn3; d.niin3 = s.niin3; d.flags = s.flags; d.land = s.land;
}

template <class T> const TempoConsts<T>& consts_of(const tempo_ctx* c);
template <> const TempoConsts<double>& consts_of<double>(const tempo_ctx* c) { return c->c64; }
template <> const TempoConsts<float>& consts_of<float>(const tempo_ctx* c) { return c->c32; }

// Packed (value, tangent) copies of a state and the step's scratch for Dual<T, 1>.
template <class T>
struct DualStep {
  using D1 = Dual<T, 1>;
  StepArgs<D1> a{};
  D1* f[19] = {};  // t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb
  D1* dg[15] = {};
  size_t ext = 0, n2 = 0, n3 = 0;

  int setup(tempo_ctx* c, const StepArgs<T>& ap, const Bounds& b, const RunArrays<T>& X,
            const RunArrays<T>* dX, DevBufs& B, cudaStream_t s) {
    copy_scalars(a, ap);
    ext = (size_t)(b.ime - b.ims + 1) * (b.kme - b.kms + 1) * (b.jme - b.jms + 1);
    n2 = (size_t)ap.ti * ap.tj;
    n3 = n2 * ap.nz;
    const T* xs[19] = {X.t, X.th, X.pii, X.p, X.w, X.dz, X.qv, X.qc, X.qr, X.qi, X.qs, X.qg,
                       X.ni, X.nr, X.nc, X.nwfa, X.nifa, X.ng, X.qb};
    const T* ds[19] = {};
    if (dX) {
      const T* d2[19] = {dX->t, dX->th, nullptr, nullptr, nullptr, nullptr, dX->qv, dX->qc,
                         dX->qr, dX->qi, dX->qs, dX->qg, dX->ni, dX->nr, dX->nc, nullptr,
                         nullptr, dX->ng, dX->qb};
      for (int i = 0; i < 19; i++) ds[i] = d2[i];
    }
    for (int i = 0; i < 19; i++) {
      if (!xs[i]) continue;
      if (!(f[i] = B.alloc<D1>(ext))) return fail(TEMPO_ERR_NOMEM, "derivative step: state copy");
      if (DerivOps<T>::pack(f[i], xs[i], ds[i], (long)ext, s) != cudaSuccess)
        return fail(TEMPO_ERR_CUDA, "derivative step: pack");
    }
    a.t = f[0]; a.th = f[1]; a.pii = f[2]; a.p = f[3]; a.w = f[4]; a.dz = f[5]; a.qv = f[6];
    a.qc = f[7]; a.qr = f[8]; a.qi = f[9]; a.qs = f[10]; a.qg = f[11]; a.ni = f[12]; a.nr = f[13];
    a.nc = f[14]; a.nwfa = f[15]; a.nifa = f[16]; a.ng = f[17]; a.qb = f[18];
    T* const* dp = (T* const*)&ap.rain_precip;  // the 15 diagnostic pointers, in order
    D1** dd = (D1**)&a.rain_precip;
    for (int i = 0; i < 15; i++) {
      if (!dp[i]) continue;
      if (!(dg[i] = B.alloc<D1>(i < 8 ? n2 : n3))) return fail(TEMPO_ERR_NOMEM, "derivative step: diagnostics");
      if (DerivOps<T>::pack(dg[i], nullptr, nullptr, (long)(i < 8 ? n2 : n3), s) != cudaSuccess)
        return fail(TEMPO_ERR_CUDA, "derivative step: pack");
      dd[i] = dg[i];
    }
    const size_t npad = (size_t)a.ncol_pad, nzs = (size_t)a.nz;
    if (!(a.sd = B.alloc<D1>((size_t)SD_N * nzs * npad)) || !(a.sr = B.alloc<D1>((size_t)SR_N * nzs * npad)) ||
        !(a.sc = B.alloc<D1>((size_t)SC_N * npad)) || !(a.act = B.alloc<int>(npad)) ||
        !(a.pmask = B.alloc<uint8_t>(nzs * npad)) || !(a.cmask = B.alloc<uint8_t>(npad)) ||
        !(a.hgt = B.alloc<T>(nzs * npad)) || !(a.nact = B.alloc<unsigned>(2)))
      return fail(TEMPO_ERR_NOMEM, "derivative step: scratch");
    if (c->points_order && !(a.ord = B.alloc<unsigned>(nzs * npad)))
      return fail(TEMPO_ERR_NOMEM, "derivative step: point order");
    a.stats = c->d_stats;
    if (cudaMemsetAsync(a.nact, 0, 2 * sizeof(unsigned), s) != cudaSuccess ||
        cudaMemsetAsync(c->d_stats, 0, 8 * sizeof(unsigned long long), s) != cudaSuccess)
      return fail(TEMPO_ERR_CUDA, "derivative step: counters");
    return TEMPO_OK;
  }
};

template <class T>
int tl_dev(tempo_ctx* c, const tempo_cfgs_t* cfg, double dt, int itimestep, tempo_state_t* x,
           tempo_state_t* dx, tempo_diags_t* dgs, tempo_diags_t* ddg, const Bounds& b, cudaStream_t s) {
  if (!x) return fail(TEMPO_ERR_ARG, "NULL state");
  const RunArrays<T> X = arrays_of<T>(x);
  StepArgs<T> ap;
  if (int rc = build_args(c, cfg, dt, itimestep, X, b, dgs, ap)) return rc;
  if (ap.flags & (F_SEMI | F_MELT | F_MLNC))
    return fail(TEMPO_ERR_UNSUPPORTED, "derivatives of the semi-Lagrangian sedimentation, the "
                "melting-layer reflectivity and the ML cloud number are not implemented by this library");
  if (cfg->max_hail_diameter_flag) ap.mhd_sfc = ap.mhd_col = nullptr;  // not differentiable
  if (int rc = check_current_device(c)) return rc;
  DevBufs B;
  DualStep<T> st;
  const RunArrays<T> DX = dx ? arrays_of<T>(dx) : RunArrays<T>{};
  if (int rc = st.setup(c, ap, b, X, dx ? &DX : nullptr, B, s)) return rc;
  IslandConsts<Dual<T, 1>> ci;
  make_island_consts(c->c64, &ci);
  CUDA_TRY(DerivOps<T>::tl_step(st.a, tables_of<T>(c), consts_of<T>(c), ci, s, 0));
  T* xs[19] = {X.t, X.th, nullptr, nullptr, nullptr, nullptr, X.qv, X.qc, X.qr, X.qi, X.qs, X.qg,
               X.ni, X.nr, X.nc, X.nwfa, X.nifa, X.ng, X.qb};
  T* ds[19] = {};
  if (dx) {
    T* d2[19] = {DX.t, DX.th, nullptr, nullptr, nullptr, nullptr, DX.qv, DX.qc, DX.qr, DX.qi, DX.qs,
                 DX.qg, DX.ni, DX.nr, DX.nc, nullptr, nullptr, DX.ng, DX.qb};
    for (int i = 0; i < 19; i++) ds[i] = d2[i];
  }
  for (int i = 0; i < 19; i++)
    if (st.f[i] && (xs[i] || ds[i])) CUDA_TRY(DerivOps<T>::unpack(xs[i], ds[i], st.f[i], (long)st.ext, s));
  T* const* dp = (T* const*)&ap.rain_precip;
  T* const* tp = ddg ? (T* const*)ddg : nullptr;
  for (int i = 0; i < 15; i++)
    if (st.dg[i]) CUDA_TRY(DerivOps<T>::unpack(dp[i], tp ? tp[i] : nullptr, st.dg[i],
                                               (long)(i < 8 ? st.n2 : st.n3), s));
  CUDA_TRY(cudaStreamSynchronize(s));
  c->last_cols = ap.ncol;
  c->launches = kStepLaunches + (c->points_order ? kOrderLaunches : 0);
  return TEMPO_OK;
}

template <class T>
int adjoint_dev(tempo_ctx* c, const tempo_cfgs_t* cfg, double dt, int itimestep, const tempo_state_t* x,
                tempo_state_t* lam, const tempo_diags_t* ldg, const Bounds& b, cudaStream_t s) {
  if (!x || !lam) return fail(TEMPO_ERR_ARG, "NULL state or adjoint");
  const RunArrays<T> X = arrays_of<T>(x);
  StepArgs<T> ap;
  if (int rc = build_args(c, cfg, dt, itimestep, X, b, nullptr, ap)) return rc;
  if (ap.flags & (F_SEMI | F_MELT | F_MLNC))
    return fail(TEMPO_ERR_UNSUPPORTED, "derivatives of the semi-Lagrangian sedimentation, the "
                "melting-layer reflectivity and the ML cloud number are not implemented by this library");
  if (int rc = check_current_device(c)) return rc;
  DevBufs B;
  using D1 = Dual<T, 1>;
  // 1. forward trajectory on packed copies (zero tangents): prep and phase A
  DualStep<T> st;
  if (int rc = st.setup(c, ap, b, X, nullptr, B, s)) return rc;
  IslandConsts<Dual<T, 1>> ci1;
  make_island_consts(c->c64, &ci1);
  const Tables<T> TT = tables_of<T>(c);
  const TempoConsts<T>& cst = consts_of<T>(c);
  CUDA_TRY(DerivOps<T>::tl_step(st.a, TT, cst, ci1, s, 1));
  // 2. snapshots: scratch before sedimentation, state after phase A (plain values)
  const size_t npad = (size_t)ap.ncol_pad, nzs = (size_t)ap.nz;
  const size_t nsd = (size_t)SD_N * nzs * npad, nsr = (size_t)SR_N * nzs * npad;
  D1* sd_pre = B.alloc<D1>(nsd);
  D1* sr_pre = B.alloc<D1>(nsr);
  if (!sd_pre || !sr_pre) return fail(TEMPO_ERR_NOMEM, "adjoint: scratch snapshot");
  CUDA_TRY(cudaMemcpyAsync(sd_pre, st.a.sd, nsd * sizeof(D1), cudaMemcpyDeviceToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(sr_pre, st.a.sr, nsr * sizeof(D1), cudaMemcpyDeviceToDevice, s));
  StepArgs<T> aC = ap;  // phase C reads the state after phase A
  {
    const int idx[11] = {6, 7, 8, 9, 10, 11, 12, 13, 14, 17, 18};  // qv qc qr qi qs qg ni nr nc ng qb
    T** dst[11] = {&aC.qv, &aC.qc, &aC.qr, &aC.qi, &aC.qs, &aC.qg, &aC.ni, &aC.nr, &aC.nc, &aC.ng, &aC.qb};
    for (int i = 0; i < 11; i++) {
      if (!st.f[idx[i]]) {
        *dst[i] = nullptr;
        continue;
      }
      T* q = B.alloc<T>(st.ext);
      if (!q) return fail(TEMPO_ERR_NOMEM, "adjoint: state snapshot");
      CUDA_TRY(DerivOps<T>::unpack(q, nullptr, st.f[idx[i]], (long)st.ext, s));
      *dst[i] = q;
    }
  }
  // 3. sedimentation of the trajectory; its substep counts size the checkpoints
  CUDA_TRY(DerivOps<T>::tl_step(st.a, TT, cst, ci1, s, 2));
  unsigned long long sub[8];
  CUDA_TRY(cudaMemcpyAsync(sub, c->d_stats, sizeof sub, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  unsigned long long smax = 1;
  for (int i = 1; i <= 5; i++) smax = std::max(smax, sub[i]);
  SedWork W;
  W.nck = (int)((smax + 3) / 4);
  W.rows = SedWork::rows_for(W.nck, (int)nzs);
  // 4. adjoint storage
  T* lam_sd = B.alloc<T>(nsd);
  T* lam_sr = B.alloc<T>(nsr);
  T* work = B.alloc<T>((size_t)W.rows * npad);
  uint8_t* colflag = B.alloc<uint8_t>((size_t)ap.ncol);
  if (!lam_sd || !lam_sr || !work || !colflag) return fail(TEMPO_ERR_NOMEM, "adjoint: workspace");
  CUDA_TRY(cudaMemsetAsync(lam_sd, 0, nsd * sizeof(T), s));
  CUDA_TRY(cudaMemsetAsync(lam_sr, 0, nsr * sizeof(T), s));
  AdjArgs<T> j{};
  const RunArrays<T> L = arrays_of<T>(lam);
  j.lam[A_T] = L.t;
  j.lam_th = L.th;
  j.lam[A_QV] = L.qv;
  j.lam[A_QC] = L.qc;
  j.lam[A_NC] = L.nc;
  j.lam[A_QR] = L.qr;
  j.lam[A_NR] = L.nr;
  j.lam[A_QI] = L.qi;
  j.lam[A_NI] = L.ni;
  j.lam[A_QS] = L.qs;
  j.lam[A_QG] = L.qg;
  j.lam[A_NG] = L.ng;
  j.lam[A_QB] = L.qb;
  if (ldg) {
    j.lam_refl = (T*)ldg->refl10cm;
    j.lam_precip[0] = (T*)ldg->rain_precip;
    j.lam_precip[1] = (T*)ldg->ice_liquid_equiv_precip;
    j.lam_precip[2] = (T*)ldg->snow_liquid_equiv_precip;
    j.lam_precip[3] = (T*)ldg->graupel_liquid_equiv_precip;
  }
  j.lam_sd = lam_sd;
  j.lam_sr = lam_sr;
  j.colflag = colflag;
  // shared step bookkeeping of the trajectory (phase A's adjoint takes its points in
  // the trajectory's order)
  ap.ord = st.a.ord;
  for (StepArgs<T>* q : {&aC, &ap}) {
    q->act = st.a.act;
    q->nact = st.a.nact;
    q->pmask = st.a.pmask;
    q->cmask = st.a.cmask;
    q->hgt = st.a.hgt;
    q->stats = c->d_stats;
    q->sd = q->sr = q->sc = nullptr;
  }
  // the reflectivity's adjoint is read where phase C produces it
  aC.refl10cm = (cfg->refl10cm_flag && j.lam_refl) ? j.lam_refl : nullptr;
  // 5. reverse: phase C, sedimentation, phase A, early-exit columns
  j.psd = (const D1*)st.a.sd;
  j.psc = (const D1*)st.a.sc;
  IslandConsts<Dual<T, C_N>> ciC;
  make_island_consts(c->c64, &ciC);
  CUDA_TRY(DerivOps<T>::adj_final(aC, cst, ciC, j, s));
  j.psd = sd_pre;
  j.psr = sr_pre;
  CUDA_TRY(DerivOps<T>::adj_sedim(aC, j, work, W, s));
  IslandConsts<Dual<T, IN_N>> ciA;
  make_island_consts(c->c64, &ciA);
  if (ap.flags & F_HAIL) {
    CUDA_TRY(DerivOps<T>::adj_points(ap, TT, cst, ciA, j, s));
  } else {  // ng and qb are no inputs: two directions fewer
    IslandConsts<Dual<T, IN_NG>> ciA10;
    make_island_consts(c->c64, &ciA10);
    CUDA_TRY(DerivOps<T>::adj_points_nohail(ap, TT, cst, ciA10, j, s));
  }
  CUDA_TRY(DerivOps<T>::colflag(colflag, st.a.act, st.a.nact, ap.ncol, s));
  CUDA_TRY(DerivOps<T>::adj_early(ap, cst, ciA, j, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  c->last_cols = ap.ncol;
  return TEMPO_OK;
}

}  // namespace

extern "C" {

int tempo_tl_dev_c(tempo_ctx_t* c, const tempo_cfgs_t* cfg, double dt, int itimestep, int fp64,
                   tempo_state_t* x, tempo_state_t* dx, tempo_diags_t* diags, tempo_diags_t* tdiags,
                   int ims, int ime, int jms, int jme, int kms, int kme, int its, int ite, int jts,
                   int jte, int kts, int kte, void* stream) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  const Bounds b{ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte};
  cudaStream_t s = (cudaStream_t)stream;
  return fp64 ? tl_dev<double>(c, cfg, dt, itimestep, x, dx, diags, tdiags, b, s)
              : tl_dev<float>(c, cfg, dt, itimestep, x, dx, diags, tdiags, b, s);
}

int tempo_adjoint_dev_c(tempo_ctx_t* c, const tempo_cfgs_t* cfg, double dt, int itimestep, int fp64,
                        const tempo_state_t* x, tempo_state_t* lam, const tempo_diags_t* lam_diags,
                        int ims, int ime, int jms, int jme, int kms, int kme, int its, int ite,
                        int jts, int jte, int kts, int kte, void* stream) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  const Bounds b{ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte};
  cudaStream_t s = (cudaStream_t)stream;
  return fp64 ? adjoint_dev<double>(c, cfg, dt, itimestep, x, lam, lam_diags, b, s)
              : adjoint_dev<float>(c, cfg, dt, itimestep, x, lam, lam_diags, b, s);
}

int tempo_run_batch_dev_f32_c(tempo_ctx_t* c, const tempo_cfgs_t* cfg, int ndomains,
                              const tempo_domain_t* domains, void* stream) {
  return run_batch(c, cfg, ndomains, domains, (cudaStream_t)stream);
}

int tempo_aerosol_surface_emissions_dev_c(tempo_ctx_t* c, double dt, double* nwfa,
                                          const double* nwfa2d, int ims, int ime, int jms, int jme,
                                          int kms, int kme, int kts, void* stream) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  if (!nwfa || !nwfa2d) return fail(TEMPO_ERR_ARG, "NULL array");
  if (ime < ims || jme < jms || kme < kms || kts < kms || kts > kme)
    return fail(TEMPO_ERR_ARG, "bad bounds");
  if (int rc = check_current_device(c)) return rc;
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  CUDA_TRY(launch_surface_emissions(nwfa, nwfa2d, ime - ims + 1, kme - kms + 1, jme - jms + 1,
                                    kts - kms, dt, s));
  return TEMPO_OK;
}

int tempo_build_tables_c(tempo_ctx_t* c, float* ms) {
  if (!c) return fail(TEMPO_ERR_STATE, "NULL context");
  int rc = build_tables_gpu(c, ms);
  if (rc) return rc;
  return make_f32_tables(c);
}

int tempo_get_table_c(tempo_ctx_t* c, const char* name, double* host_out, long count, long* needed) {
  if (!c || !name) return fail(TEMPO_ERR_ARG, "NULL argument");
  struct E {
    const char* n;
    const double* aos;
    long cnt;
    int nfam, slot;
  } tab[] = {
      {"t_efrw", c->t64.t_efrw, (long)nbr * nbc, 1, 0},
      {"t_efsw", c->t64.t_efsw, (long)nbs * nbc, 1, 0},
      {"tpc_wev", c->t64.tpc_wev, (long)nbc * ntb_c * nbc, 1, 0},
      {"tnc_wev", c->t64.tnc_wev, (long)nbc * ntb_c * nbc, 1, 0},
      {"tps_iaus", c->t64.tps_iaus, (long)ntb_i * ntb_i1, 1, 0},
      {"tni_iaus", c->t64.tni_iaus, (long)ntb_i * ntb_i1, 1, 0},
      {"tpi_ide", c->t64.tpi_ide, (long)ntb_i * ntb_i1, 1, 0},
      {"tcg_racg", c->t64.qg, QG_COUNT, 5, 0},   {"tmr_racg", c->t64.qg, QG_COUNT, 5, 1},
      {"tcr_gacr", c->t64.qg, QG_COUNT, 5, 2},   {"tnr_racg", c->t64.qg, QG_COUNT, 5, 3},
      {"tnr_gacr", c->t64.qg, QG_COUNT, 5, 4},   {"tcs_racs1", c->t64.qs, QS_COUNT, 12, 0},
      {"tmr_racs1", c->t64.qs, QS_COUNT, 12, 1}, {"tcs_racs2", c->t64.qs, QS_COUNT, 12, 2},
      {"tmr_racs2", c->t64.qs, QS_COUNT, 12, 3}, {"tcr_sacr1", c->t64.qs, QS_COUNT, 12, 4},
      {"tms_sacr1", c->t64.qs, QS_COUNT, 12, 5}, {"tcr_sacr2", c->t64.qs, QS_COUNT, 12, 6},
      {"tms_sacr2", c->t64.qs, QS_COUNT, 12, 7}, {"tnr_racs1", c->t64.qs, QS_COUNT, 12, 8},
      {"tnr_racs2", c->t64.qs, QS_COUNT, 12, 9}, {"tnr_sacr1", c->t64.qs, QS_COUNT, 12, 10},
      {"tnr_sacr2", c->t64.qs, QS_COUNT, 12, 11}, {"tpi_qrfz", c->t64.qrfz, QRFZ_COUNT, 4, 0},
      {"tni_qrfz", c->t64.qrfz, QRFZ_COUNT, 4, 1}, {"tpg_qrfz", c->t64.qrfz, QRFZ_COUNT, 4, 2},
      {"tnr_qrfz", c->t64.qrfz, QRFZ_COUNT, 4, 3}, {"tpi_qcfz", c->t64.qcfz, QCFZ_COUNT, 2, 0},
      {"tni_qcfz", c->t64.qcfz, QCFZ_COUNT, 2, 1}};
  for (auto& t : tab) {
    if (std::strcmp(t.n, name)) continue;
    if (needed) *needed = t.cnt;
    if (!host_out) return TEMPO_OK;
    if (count < t.cnt) return fail(TEMPO_ERR_ARG, "buffer for %s holds %ld < %ld", name, count, t.cnt);
    double* tmp = nullptr;
    if (int rc = dev_alloc(&tmp, (size_t)t.cnt)) return rc;
    cudaError_t e = aos_gather(tmp, t.aos, t.cnt, t.nfam, t.slot, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_out, tmp, t.cnt * 8, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return fail(TEMPO_ERR_CUDA, "get_table: %s", cudaGetErrorString(e));
    return TEMPO_OK;
  }
  return fail(TEMPO_ERR_ARG, "unknown table '%s'", name);
}

int tempo_write_table_c(tempo_ctx_t* c, const char* name, const char* path) {
  if (!c || !name || !path) return fail(TEMPO_ERR_ARG, "NULL argument");
  const char* fz[] = {"tpi_qrfz", "tni_qrfz", "tpg_qrfz", "tnr_qrfz", "tpi_qcfz", "tni_qcfz"};
  const char* qs[] = {"tcs_racs1", "tmr_racs1", "tcs_racs2", "tmr_racs2", "tcr_sacr1", "tms_sacr1",
                      "tcr_sacr2", "tms_sacr2", "tnr_racs1", "tnr_racs2", "tnr_sacr1", "tnr_sacr2"};
  const char* qg[] = {"tcg_racg", "tmr_racg", "tcr_gacr", "tnr_racg", "tnr_gacr"};
  const char** arrs;
  int narr;
  if (!std::strcmp(name, "freezewater")) {
    arrs = fz;
    narr = 6;
  } else if (!std::strcmp(name, "qr_acr_qs")) {
    arrs = qs;
    narr = 12;
  } else if (!std::strcmp(name, "qr_acr_qg")) {
    arrs = qg;
    narr = 5;
  } else {
    return fail(TEMPO_ERR_ARG, "unknown table family '%s'", name);
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(TEMPO_ERR_ARG, "cannot create %s", path);
  std::vector<double> buf;
  for (int a = 0; a < narr; a++) {
    long n = 0;
    tempo_get_table_c(c, arrs[a], nullptr, 0, &n);
    buf.resize(n);
    int rc = tempo_get_table_c(c, arrs[a], buf.data(), n, nullptr);
    if (rc) {
      std::fclose(f);
      return rc;
    }
    if (host_little()) bswap8(buf.data(), n);
    if ((long)std::fwrite(buf.data(), 8, n, f) != n) {
      std::fclose(f);
      return fail(TEMPO_ERR_ARG, "short write to %s", path);
    }
  }
  std::fclose(f);
  return TEMPO_OK;
}

int tempo_last_stats_c(tempo_ctx_t* c, long out[8]) {
  if (!c || !out) return fail(TEMPO_ERR_ARG, "NULL argument");
  unsigned long long s[8] = {0};
  CUDA_TRY(cudaSetDevice(c->device));
  CUDA_TRY(cudaDeviceSynchronize());  // runs may be enqueued on caller streams
  CUDA_TRY(cudaMemcpy(s, c->d_stats, sizeof s, cudaMemcpyDeviceToHost));
  out[0] = c->last_cols;
  out[1] = (long)s[0];
  for (int i = 0; i < 5; i++) out[2 + i] = (long)s[1 + i];
  out[7] = c->launches;
  return TEMPO_OK;
}

}  // extern "C"
