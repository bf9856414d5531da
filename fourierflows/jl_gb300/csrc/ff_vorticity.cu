// Host side of the fused 2D vorticity path: problem descriptors, work lists, launch
// geometry, CUDA-graph capture of whole steps and the tile/radix autotuner.
#include <string.h>

#include <algorithm>
#include <map>
#include <tuple>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "ff_plan.cuh"
#include "ff_vort_launch.cuh"
#include "ff_vorticity.cuh"

using namespace ff;

namespace {

struct Geom {
  int tla = 0, tlc = 0, tlr = 0;   // tile widths of passes A, C and rows per CTA of pass B
                                   // (register path: lines per CTA of the largest problem)
  int tha = 0, thb = 0, thc = 0;   // threads per CTA
  size_t sma = 0, smb = 0, smc = 0;
  int ga = 0, gb = 0, gc = 0;      // grid sizes
  int radix_variant = 0;           // generic path: 0 radix-8 first, 1 radix-4 first, 2 small radix first
  bool reg = false;                // register-resident power-of-two kernels
  bool split_c = false;            // register path, unfused pass C: kept tiles split by field
};

int pow2_floor(int v) {
  int p = 1;
  while (p * 2 <= v) p *= 2;
  return p;
}

// factorisation variants explored by the autotuner
bool factorize_variant(int n, int variant, LinePlan& P) {
  if (!factorize(n, P)) return false;
  if (variant == 1) {
    // prefer radix 4: split each 8 into 4 * 2 pairs -> 8*8 = 4*4*4
    int twos = 0, rest[FF_MAX_STAGES], nr = 0;
    for (int s = 0; s < P.nst; ++s) {
      int r = P.radix[s];
      if (r == 8) twos += 3;
      else if (r == 4) twos += 2;
      else if (r == 2) twos += 1;
      else rest[nr++] = r;
    }
    P.nst = 0;
    while (twos >= 2) { P.radix[P.nst++] = 4; twos -= 2; }
    if (twos) P.radix[P.nst++] = 2;
    for (int i = 0; i < nr; ++i) P.radix[P.nst++] = rest[i];
  } else if (variant == 2) {
    std::reverse(P.radix, P.radix + P.nst);
  }
  return true;
}

int round32(int t, int lo, int hi) {
  t = ((t + 31) / 32) * 32;
  return std::max(lo, std::min(hi, t));
}

}  // namespace

struct ff_vort {
  int prec = FF_F64, stepper = FF_STEP_ETDRK4, dev = 0;
  int64_t nprob = 0;
  double dt = 0;
  bool filtered = false;
  std::vector<ff_vort_problem> host;  // as given
  int max_nx = 0, max_ny = 0, max_nkd = 0;
  // device allocations
  void* d_probs = nullptr;     // VortProb<T>[nprob]
  void* d_calc_prob = nullptr; // VortProb<T>[1] for ff_vort_calcN
  void* d_work_a = nullptr;
  void* d_work_b = nullptr;
  void* d_work_c = nullptr;
  void* d_calc_work = nullptr;  // single-problem work lists (a | b | c)
  void* d_inputs = nullptr;     // const cx<T>*[5][nprob]: pass-A inputs per substep
  void* d_calc_input = nullptr;
  int nwork_a = 0, nwork_b = 0, nwork_c = 0;
  int nwork_c_kept = 0;         // pass C: the kept-column tiles, a prefix of the work list
  int split_mode = -1;          // pass C split by field: -1 automatic, 0 off, 1 on
  void* d_cnt = nullptr;        // its arrival counters, one per kept column tile
  std::vector<void*> tables;    // twiddle tables
  void* d_W = nullptr;
  void* d_Q = nullptr;
  Geom g;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  bool use_graph = true;
  std::vector<unsigned char> calc_host;  // staging for ff_vort_calcN descriptor + work
  // ff_vort_calcN_bind slots: a descriptor, work lists and input pointer each, staged once
  struct CalcSlot {
    void* d = nullptr;
    int nwa = 0, nwb = 0, nwc = 0;
    uint64_t gen = 0;
  };
  std::vector<CalcSlot> slots;
  uint64_t gen = 0;  // geometry generation: a rebuild invalidates the bound slots
  std::vector<unsigned char> host_desc;  // host copy of the device descriptors
  size_t calc_cap = 0;
};

namespace {

template <typename T> size_t elem() { return sizeof(cx<T>); }

bool reg_capable(const ff_vort* h) {
  const char* gen = getenv("FF_VORT_GENERIC");
  if (gen && gen[0] == '1') return false;
  for (const auto& q : h->host)
    if (!regfft_ok((int)q.ny) || !regfft_ok((int)(q.nx / 2)) || q.nx / 2 > 2048) return false;
  return true;
}

// row pitch of W and Q in elements: rows start on 16-byte boundaries for the bulk copies
static int64_t wq_pitch(int64_t nkd, size_t es) {
  const int64_t m = 16 / (int64_t)es;
  return (nkd + m - 1) / m * m;
}

template <typename T> Geom choose_geom_reg(const ff_vort* h, int tla, int tlc, int tlr) {
  Geom g;
  g.reg = true;
  const size_t es = elem<T>();
  const int ny = h->max_ny, hx = h->max_nx / 2;
  const bool f64 = sizeof(T) == 8;
  g.tla = tla > 0 ? tla : (f64 ? 2 : 4);
  g.tlc = tlc > 0 ? tlc : (f64 ? 2 : 4);
  g.tlr = tlr > 0 ? tlr : (f64 ? 2 : 4);
  auto threads = [](int lines, int n, int cap) {
    int t = pow2_floor(std::max(1, lines)) * (n / 8);
    t = std::max(t, n / 8);
    t = std::max(t, 32);
    while (t > cap && t > n / 8) t /= 2;
    return t;
  };
  g.tha = threads(g.tla, ny, 512);
  g.thc = threads(g.tlc, ny, 512);
  g.thb = threads(g.tlr, hx, FF_LB_B_THREADS);
  g.tla = g.tha * 8 / ny;
  g.tlc = g.thc * 8 / ny;
  g.tlr = g.thb * 8 / hx;
  g.sma = 9 * (size_t)AFields<T>::value * g.tha * es;
  // pass C's exchanges: its own two fields, or the fused pass A's fields if more
  g.smc = (size_t)std::max(2, FuseA<T>::value ? AFields<T>::value : 2) * 9 * (size_t)g.thc * es;
  size_t smb = 0;
  const int sh = f64 ? 3 : 4;
  for (const auto& q : h->host) {
    const int H = (int)(q.nx / 2);
    const size_t rows = (size_t)g.thb * 8 / H;
    smb = std::max(smb, 3 * rows * (size_t)(H + (H >> sh) + 1) * es);
  }
  g.smb = smb;
  // Pass C split by field where it runs unfused: twice the work items for a grid with
  // few kept column tiles per SM (one 1024^2 problem: 342 tiles of one column on 152 SMs)
  if (!FuseA<T>::value && g.thc <= FF_SPLIT_C_THREADS) {
    int64_t tiles = 0;
    for (const auto& q : h->host) tiles += ceil_div(q.nkd, std::max(1, g.thc * 8 / (int)q.ny));
    g.split_c = h->split_mode == 1 || (h->split_mode == -1 && tiles < 8 * (int64_t)sm_count());
  }
  return g;
}

template <typename T> Geom choose_geom(const ff_vort* h, int tla, int tlc, int tlr, int variant) {
  if (reg_capable(h)) return choose_geom_reg<T>(h, tla, tlc, tlr);
  Geom g;
  const int ny = h->max_ny, hx = h->max_nx / 2;
  const size_t es = elem<T>();
  g.tla = tla > 0 ? tla : (sizeof(T) == 8 ? 2 : 4);
  g.tlc = tlc > 0 ? tlc : (sizeof(T) == 8 ? 1 : 2);
  g.tlr = tlr > 0 ? tlr : (sizeof(T) == 8 ? 2 : 4);
  while (g.tla > 1 && 2 * (size_t)g.tla * ny * es > 110 * 1024) g.tla /= 2;
  while (g.tlc > 1 && 4 * (size_t)g.tlc * ny * es > 110 * 1024) g.tlc /= 2;
  while (g.tlr > 1 && 4 * (size_t)g.tlr * rows_stride(hx, (int)es) * es > 110 * 1024) g.tlr /= 2;
  g.sma = 2 * (size_t)g.tla * ny * es;
  g.smc = 4 * (size_t)g.tlc * ny * es;
  g.smb = 4 * (size_t)g.tlr * rows_stride(hx, (int)es) * es;
  g.tha = round32(g.tla * ny / 8, 64, 512);
  g.thc = round32(2 * g.tlc * ny / 8, 64, 512);
  g.thb = round32(g.tlr * hx / 4, 64, 512);
  g.radix_variant = variant;
  return g;
}

template <typename T> int grid_for(const void* k, int threads, size_t smem, int nwork) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int cap = per_sm * sm_count();
  return std::max(1, std::min(nwork, cap));
}

template <typename T> int build(ff_vort* h, const Geom& geom) {
  // descriptors, twiddles and work lists for the current geometry
  for (void* p : h->tables) cudaFree(p);
  h->tables.clear();
  std::vector<VortProb<T>> probs(h->nprob);
  std::vector<WorkItem> wa, wb, wc;
  const size_t es = elem<T>();
  int64_t woff = 0, coff = 0;
  std::map<std::tuple<const void*, const void*, int, int>, const void*> scaled;
  if (h->d_cnt) { cudaFree(h->d_cnt); h->d_cnt = nullptr; }
  if (geom.split_c) {
    int64_t tiles = 0;
    for (const auto& q : h->host) tiles += ceil_div(q.nkd, std::max(1, geom.thc * 8 / (int)q.ny));
    FF_CUDA(cudaMalloc(&h->d_cnt, sizeof(unsigned) * tiles));
    FF_CUDA(cudaMemset(h->d_cnt, 0, sizeof(unsigned) * tiles));
  }
  for (int64_t i = 0; i < h->nprob; ++i) {
    const ff_vort_problem& q = h->host[i];
    VortProb<T>& P = probs[i];
    memset(&P, 0, sizeof(P));
    P.nx = (int)q.nx;
    P.ny = (int)q.ny;
    P.nkr = (int)(q.nx / 2 + 1);
    P.nkd = (int)q.nkd;
    P.nkp = (int)wq_pitch(q.nkd, elem<T>());
    P.la = (int)q.la;
    P.lb = (int)q.lb;
    const double s = 1.0 / ((double)q.nx * (double)q.ny);
    P.scale2 = (T)(s * s);
    if (!factorize_variant(P.nx / 2, geom.radix_variant, P.Px) || !factorize_variant(P.ny, geom.radix_variant, P.Py)) {
      set_error("ff_vort: grid %lld x %lld has a prime factor above %d", (long long)q.nx, (long long)q.ny,
                FF_MAX_GENERIC_RADIX);
      return FF_ERR_UNSUPPORTED;
    }
    std::vector<double> t;
    void* d = nullptr;
    host_twiddles(P.nx / 2, t);
    if (int st = upload_table(t, sizeof(T) == 8 ? FF_F64 : FF_F32, &d)) return st;
    h->tables.push_back(d);
    P.twx = (const cx<T>*)d;
    host_twiddles(P.ny, t);
    if (int st = upload_table(t, sizeof(T) == 8 ? FF_F64 : FF_F32, &d)) return st;
    h->tables.push_back(d);
    P.twy = (const cx<T>*)d;
    host_real_twiddles(P.nx, t);
    if (int st = upload_table(t, sizeof(T) == 8 ? FF_F64 : FF_F32, &d)) return st;
    h->tables.push_back(d);
    P.rtw = (const cx<T>*)d;
    P.kr = (const T*)q.kr;
    P.l = (const T*)q.l;
    P.invK = (const T*)q.invKrsq;
    if (geom.reg) {
      // kr and l times scale2 / 2 (a power of two: exact), one table per distinct
      // (kr, l, size) among the problems
      const auto key = std::make_tuple(q.kr, q.l, P.nx, P.ny);
      auto hit = scaled.find(key);
      if (hit == scaled.end()) {
        std::vector<T> kr(P.nkr), l(P.ny);
        FF_CUDA(cudaMemcpy(kr.data(), q.kr, kr.size() * sizeof(T), cudaMemcpyDeviceToHost));
        FF_CUDA(cudaMemcpy(l.data(), q.l, l.size() * sizeof(T), cudaMemcpyDeviceToHost));
        const double ps = 0.5 * s * s;
        std::vector<double> ts;
        for (T x : kr) ts.push_back((double)x * ps);
        for (T x : l) ts.push_back((double)x * ps);
        if (ts.size() % 2) ts.push_back(0.0);  // the table uploads (re, im) pairs
        if (int st = upload_table(ts, sizeof(T) == 8 ? FF_F64 : FF_F32, &d)) return st;
        h->tables.push_back(d);
        hit = scaled.emplace(key, (const void*)d).first;
      }
      P.krs = (const T*)hit->second;
      P.ls = P.krs + P.nkr;
    }
    P.W = (cx<T>*)h->d_W + woff * 3;
    P.Q = (cx<T>*)h->d_Q + woff * 2;
    woff += (int64_t)P.nkp * P.ny;
    P.sol = (cx<T>*)q.sol;
    P.filter = (const T*)q.filter;
    if (h->stepper == FF_STEP_ETDRK4) {
      P.eL = (const T*)q.coef[0];
      P.eh = (const T*)q.coef[1];
      P.zc = (const T*)q.coef[2];
      P.al = (const T*)q.coef[3];
      P.be = (const T*)q.coef[4];
      P.ga = (const T*)q.coef[5];
    } else {
      P.L = (const T*)q.coef[0];
    }
    if (h->stepper == FF_STEP_ETDRK4) {
      P.s1 = (cx<T>*)q.buf[0];
      P.s2 = (cx<T>*)q.buf[1];
      P.n1 = (cx<T>*)q.buf[2];
      P.n2 = (cx<T>*)q.buf[3];
      P.n3 = (cx<T>*)q.buf[4];
    } else if (h->stepper == FF_STEP_RK4) {
      P.s1 = (cx<T>*)q.buf[0];
      P.n1 = (cx<T>*)q.buf[1];
      P.n2 = (cx<T>*)q.buf[2];
      P.n3 = (cx<T>*)q.buf[3];
    } else {
      P.s1 = (cx<T>*)q.buf[0];
    }
    // tile widths: fixed on the generic path; on the register path a CTA holds
    // threads*8 elements, i.e. threads*8/N lines of this problem's length N
    const int wa_ = geom.reg ? geom.tha * 8 / P.ny : geom.tla;
    const int wb_ = geom.reg ? geom.thb * 8 / (P.nx / 2) : geom.tlr;
    const int wc_ = geom.reg ? geom.thc * 8 / P.ny : geom.tlc;
    const int ta = (int)ceil_div(P.nkd, wa_);
    const int afields = geom.reg && AFields<T>::value == 3 ? 1 : 3;  // work items per tile
    for (int f = 0; f < afields; ++f)
      for (int tt = 0; tt < ta; ++tt) wa.push_back({(int)i, tt, f, 0});
    const int tb = (int)ceil_div(P.ny, wb_);
    for (int tt = 0; tt < tb; ++tt) wb.push_back({(int)i, tt, 0, 0});
    const int tc = (int)ceil_div(P.nkr, wc_);
    for (int tt = 0; tt < tc; ++tt) {
      wc.push_back({(int)i, tt, 0, 0});
      if (geom.split_c && tt * wc_ < P.nkd) wc.push_back({(int)i, tt, 1, 0});
    }
    if (geom.split_c) {
      P.cnt = (unsigned*)h->d_cnt + coff;
      coff += ceil_div(P.nkd, wc_);
    }
  }
  // longest work first helps the persistent grid balance uneven sizes
  auto by_size = [&](const WorkItem& a, const WorkItem& b) {
    return (int64_t)probs[a.prob].nx * probs[a.prob].ny > (int64_t)probs[b.prob].nx * probs[b.prob].ny;
  };
  std::stable_sort(wa.begin(), wa.end(), by_size);
  // Pass B walks problems of equal size in the reverse order of passes A and C, so that
  // it starts on the problems whose W the column pass wrote last (still in L2 when an
  // ensemble's W is larger than L2), and pass C starts on the Q that B wrote last.
  auto by_size_rev = [&](const WorkItem& a, const WorkItem& b) {
    const int64_t sa = (int64_t)probs[a.prob].nx * probs[a.prob].ny, sb = (int64_t)probs[b.prob].nx * probs[b.prob].ny;
    if (sa != sb) return sa > sb;
    return a.prob > b.prob;
  };
  std::stable_sort(wb.begin(), wb.end(), by_size_rev);
  // pass C: tiles of kept columns first (largest problems first), then aliased columns
  auto kept_then_size = [&](const WorkItem& a, const WorkItem& b) {
    const int wa_c = geom.reg ? geom.thc * 8 / probs[a.prob].ny : geom.tlc;
    const int wb_c = geom.reg ? geom.thc * 8 / probs[b.prob].ny : geom.tlc;
    const bool ka = a.tile * wa_c < probs[a.prob].nkd, kb = b.tile * wb_c < probs[b.prob].nkd;
    if (ka != kb) return ka;
    return by_size(a, b);
  };
  std::stable_sort(wc.begin(), wc.end(), kept_then_size);
  h->nwork_c_kept = 0;
  for (const WorkItem& it : wc) {
    const int w_c = geom.reg ? geom.thc * 8 / probs[it.prob].ny : geom.tlc;
    if (it.tile * w_c < probs[it.prob].nkd) ++h->nwork_c_kept;
  }
  for (void** p : {&h->d_probs, &h->d_work_a, &h->d_work_b, &h->d_work_c, &h->d_inputs})
    if (*p) { cudaFree(*p); *p = nullptr; }
  h->host_desc.resize(sizeof(VortProb<T>) * h->nprob);
  memcpy(h->host_desc.data(), probs.data(), h->host_desc.size());
  FF_CUDA(cudaMalloc(&h->d_probs, sizeof(VortProb<T>) * h->nprob));
  FF_CUDA(cudaMemcpy(h->d_probs, probs.data(), sizeof(VortProb<T>) * h->nprob, cudaMemcpyHostToDevice));
  FF_CUDA(cudaMalloc(&h->d_work_a, sizeof(WorkItem) * wa.size()));
  FF_CUDA(cudaMalloc(&h->d_work_b, sizeof(WorkItem) * wb.size()));
  FF_CUDA(cudaMalloc(&h->d_work_c, sizeof(WorkItem) * wc.size()));
  FF_CUDA(cudaMemcpy(h->d_work_a, wa.data(), sizeof(WorkItem) * wa.size(), cudaMemcpyHostToDevice));
  FF_CUDA(cudaMemcpy(h->d_work_b, wb.data(), sizeof(WorkItem) * wb.size(), cudaMemcpyHostToDevice));
  FF_CUDA(cudaMemcpy(h->d_work_c, wc.data(), sizeof(WorkItem) * wc.size(), cudaMemcpyHostToDevice));
  h->nwork_a = (int)wa.size();
  h->nwork_b = (int)wb.size();
  h->nwork_c = (int)wc.size();
  // pass-A input of each substep: sol, then the stepper's intermediate states
  std::vector<const cx<T>*> in(5 * h->nprob);
  for (int64_t i = 0; i < h->nprob; ++i) {
    const VortProb<T>& P = probs[i];
    const cx<T>* seq_etd[5] = {P.sol, P.s1, P.s2, P.s2, P.sol};
    const cx<T>* seq_rk[5] = {P.sol, P.s1, P.s1, P.s1, P.sol};
    for (int k = 0; k < 5; ++k) {
      const cx<T>* p = P.sol;
      if (h->stepper == FF_STEP_ETDRK4) p = seq_etd[k];
      else if (h->stepper == FF_STEP_RK4) p = seq_rk[k];
      in[k * h->nprob + i] = p;
    }
  }
  FF_CUDA(cudaMalloc(&h->d_inputs, sizeof(void*) * in.size()));
  FF_CUDA(cudaMemcpy(h->d_inputs, in.data(), sizeof(void*) * in.size(), cudaMemcpyHostToDevice));
  h->g = geom;
  const void* ka = vort_kernel_a<T>(geom.reg);
  const void* kb = vort_kernel_b<T>(geom.reg);
  if (int st = ensure_smem(ka, geom.sma)) return st;
  if (int st = ensure_smem(kb, geom.smb)) return st;
  for (int e = 0; e < kNumEpilogues; ++e)
    for (bool fuse : {false, true})
      for (bool split : {false, true})
        if (int st = ensure_smem(vort_kernel_c<T>(geom.reg, e, fuse, split), geom.smc)) return st;
  h->g.ga = grid_for<T>(ka, geom.tha, geom.sma, h->nwork_a);
  h->g.gb = grid_for<T>(kb, geom.thb, geom.smb, h->nwork_b);
  h->g.gc = grid_for<T>(vort_kernel_c<T>(geom.reg, EPI_ETD1, geom.reg && FuseA<T>::value, geom.split_c), geom.thc,
                        geom.smc, h->nwork_c);
  if (h->exec) { cudaGraphExecDestroy(h->exec); h->exec = nullptr; }
  if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
  ++h->gen;
  return FF_OK;
}

// launches of one pass over a descriptor array and work list (generic or register path);
// the kernels themselves are instantiated in ff_vort_launch_f32.cu / _f64.cu
template <typename T>
int launch_a(const ff_vort* h, const void* probs, const void* work, int nwork, int grid, const void* inputs,
             cudaStream_t s) {
  return vort_launch_a<T>(PassLaunch{grid, h->g.tha, h->g.sma, h->g.tla, h->g.reg}, probs, work, nwork, inputs, s);
}

template <typename T>
int launch_b(const ff_vort* h, const void* probs, const void* work, int nwork, int grid, cudaStream_t s) {
  return vort_launch_b<T>(PassLaunch{grid, h->g.thb, h->g.smb, h->g.tlr, h->g.reg}, probs, work, nwork, s);
}

// split: the work list holds the kept tiles split by field (the step's own list; the
// single-problem calcN! list is never split)
template <typename T, int EPI>
int launch_c(const ff_vort* h, const void* probs, const void* work, int nwork, int grid, EpiScalars<T> S,
             cudaStream_t s, bool fuse = false, bool split = false) {
  const EpiArgs a{(double)S.c, (double)S.b, (double)S.dt, S.first, S.use_filter};
  PassLaunch L{grid, h->g.thc, h->g.smc, h->g.tlc, h->g.reg};
  L.fuse = fuse;
  L.split = split;
  return vort_launch_c<T>(L, EPI, probs, work, nwork, a, s);
}

// One substep's calcN! with epilogue EPI on all problems; `inputs` = pass-A sources.
// On the register path the substep's pass A ran already, fused into the previous
// substep's pass C (first = false), and pass C runs the next substep's pass A unless
// this is the step's last substep (last).
// an NVTX range over one substep's launches (host side: visible when the step is enqueued
// launch by launch, FF_NO_GRAPH=1; a graph replay is one range, see ff_vort_step)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

constexpr const char* kSubstepName[kNumEpilogues] = {"calcN",        "ETDRK4 substep 1", "ETDRK4 substep 2",
                                                     "ETDRK4 substep 3", "ETDRK4 substep 4", "RK4 substep 1",
                                                     "RK4 substep 2",  "RK4 substep 3",    "RK4 substep 4",
                                                     "LSRK54 stage"};

template <typename T, int EPI>
int calc(const ff_vort* h, const void* inputs, EpiScalars<T> S, cudaStream_t s, bool first = true, bool last = true) {
  const NvtxRange range(kSubstepName[EPI]);
  const bool fused = h->g.reg && FuseA<T>::value;
  if (!fused || first)
    if (int st = launch_a<T>(h, h->d_probs, h->d_work_a, h->nwork_a, h->g.ga, inputs, s)) return st;
  if (int st = launch_b<T>(h, h->d_probs, h->d_work_b, h->nwork_b, h->g.gb, s)) return st;
  // ETDRK4 / RK4 substeps 1-3 leave the aliased columns alone on the register path (see k_vort_c_r)
  const bool kept_only = h->g.reg && (EPI == EPI_ETD1 || EPI == EPI_ETD2 || EPI == EPI_ETD3 || EPI == EPI_RK1 ||
                                      EPI == EPI_RK2 || EPI == EPI_RK3);
  return launch_c<T, EPI>(h, h->d_probs, h->d_work_c, kept_only ? h->nwork_c_kept : h->nwork_c, h->g.gc, S, s,
                          fused && !last, h->g.split_c);
}

template <typename T> int enqueue_step(const ff_vort* h, cudaStream_t s) {
  const size_t stride = sizeof(void*) * h->nprob;
  const char* in = (const char*)h->d_inputs;
  const T dt = (T)h->dt;
  EpiScalars<T> S{};
  S.use_filter = h->filtered ? 1 : 0;
  int st = FF_OK;
  if (h->stepper == FF_STEP_ETDRK4) {
    S.use_filter = 0;
    if ((st = calc<T, EPI_ETD1>(h, in, S, s, true, false))) return st;
    if ((st = calc<T, EPI_ETD2>(h, in + stride, S, s, false, false))) return st;
    if ((st = calc<T, EPI_ETD3>(h, in + 2 * stride, S, s, false, false))) return st;
    S.use_filter = h->filtered ? 1 : 0;
    return calc<T, EPI_ETD4>(h, in + 3 * stride, S, s, false, true);
  }
  if (h->stepper == FF_STEP_RK4) {
    const T half = (T)(dt / T(2));
    S.use_filter = 0;
    S.dt = dt;  // the last substep advances the aliased modes through all four stages
    S.c = half;
    if ((st = calc<T, EPI_RK1>(h, in, S, s, true, false))) return st;
    if ((st = calc<T, EPI_RK2>(h, in + stride, S, s, false, false))) return st;
    S.c = dt;
    if ((st = calc<T, EPI_RK3>(h, in + 2 * stride, S, s, false, false))) return st;
    S.c = (T)(dt / T(6));
    S.use_filter = h->filtered ? 1 : 0;
    return calc<T, EPI_RK4>(h, in + 3 * stride, S, s, false, true);
  }
  // LSRK54: Carpenter-Kennedy 2N-storage stages
  for (int i = 0; i < 5; ++i) {
    S.c = (T)h->host[0].lsrk_A[i];
    S.b = (T)h->host[0].lsrk_B[i];
    S.dt = dt;
    S.first = i == 0;
    S.use_filter = (i == 4 && h->filtered) ? 1 : 0;
    if ((st = calc<T, EPI_LS>(h, in, S, s, i == 0, i == 4))) return st;
  }
  return FF_OK;
}

int enqueue(const ff_vort* h, cudaStream_t s) {
  return h->prec == FF_F64 ? enqueue_step<double>(h, s) : enqueue_step<float>(h, s);
}

int capture(ff_vort* h) {
  cudaStream_t cs;
  FF_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  int st = FF_OK;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) st = cuda_status(e, "ff_vort: begin capture");
  if (st == FF_OK) {
    st = enqueue(h, cs);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    if (st == FF_OK && e != cudaSuccess) st = cuda_status(e, "ff_vort: end capture");
    if (st == FF_OK) {
      e = cudaGraphInstantiate(&h->exec, g, 0);
      if (e != cudaSuccess) st = cuda_status(e, "ff_vort: graph instantiate");
      h->graph = g;
    } else if (g) {
      cudaGraphDestroy(g);
    }
  }
  cudaStreamDestroy(cs);
  return st;
}

int rebuild(ff_vort* h, int tla, int tlc, int tlr, int variant) {
  if (h->prec == FF_F64) return build<double>(h, choose_geom<double>(h, tla, tlc, tlr, variant));
  return build<float>(h, choose_geom<float>(h, tla, tlc, tlr, variant));
}

void destroy(ff_vort* h) {
  if (!h) return;
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  for (void* p : h->tables) cudaFree(p);
  for (void* p : {h->d_probs, h->d_calc_prob, h->d_work_a, h->d_work_b, h->d_work_c, h->d_calc_work, h->d_inputs,
                  h->d_calc_input, h->d_W, h->d_Q, h->d_cnt})
    if (p) cudaFree(p);
  for (auto& sl : h->slots)
    if (sl.d) cudaFree(sl.d);
  delete h;
}

}  // namespace

extern "C" {

int ff_vort_create(int prec, int stepper, int filtered, double dt, int64_t nprob, const ff_vort_problem* probs,
                   ff_vort** out) {
  FF_CHECK_ARG(out && probs && nprob >= 1, "ff_vort_create: bad arguments");
  *out = nullptr;
  FF_CHECK_ARG(prec == FF_F64 || prec == FF_F32, "ff_vort_create: bad precision %d", prec);
  FF_CHECK_ARG(stepper == FF_STEP_ETDRK4 || stepper == FF_STEP_RK4 || stepper == FF_STEP_LSRK54,
               "ff_vort_create: unsupported stepper %d", stepper);
  const int64_t maxn = prec == FF_F64 ? 4096 : 8192;
  for (int64_t i = 0; i < nprob; ++i) {
    const ff_vort_problem& q = probs[i];
    FF_CHECK_ARG(q.nx >= 2 && q.ny >= 2 && q.nx % 2 == 0 && q.ny % 2 == 0,
                 "ff_vort_create: problem %lld: nx, ny must be even and >= 2", (long long)i);
    FF_CHECK_ARG(q.nx / 2 <= maxn && q.ny <= maxn, "ff_vort_create: problem %lld: grid too large", (long long)i);
    FF_CHECK_ARG(q.nkd >= 1 && q.nkd <= q.nx / 2 + 1, "ff_vort_create: problem %lld: bad nkd", (long long)i);
    FF_CHECK_ARG(q.la >= 0 && q.la <= q.lb && q.lb <= q.ny, "ff_vort_create: problem %lld: bad l range",
                 (long long)i);
    FF_CHECK_ARG(q.kr && q.l && q.invKrsq && q.sol, "ff_vort_create: problem %lld: null array", (long long)i);
    if (stepper == FF_STEP_ETDRK4) {
      for (int k = 0; k < 5; ++k) FF_CHECK_ARG(q.buf[k], "ff_vort_create: ETDRK4 needs 5 buffers");
      for (int k = 0; k < 6; ++k) FF_CHECK_ARG(q.coef[k], "ff_vort_create: ETDRK4 needs 6 coefficient arrays");
    } else if (stepper == FF_STEP_RK4) {
      for (int k = 0; k < 4; ++k) FF_CHECK_ARG(q.buf[k], "ff_vort_create: RK4 needs 4 buffers");
      FF_CHECK_ARG(q.coef[0], "ff_vort_create: RK4 needs L");
    } else {
      FF_CHECK_ARG(q.buf[0] && q.coef[0], "ff_vort_create: LSRK54 needs S2 and L");
    }
    if (filtered) FF_CHECK_ARG(q.filter, "ff_vort_create: filtered stepper without a filter");
  }
  ff_vort* h = new ff_vort();
  h->prec = prec;
  h->stepper = stepper;
  h->filtered = filtered != 0;
  h->dt = dt;
  h->nprob = nprob;
  h->host.assign(probs, probs + nprob);
  cudaGetDevice(&h->dev);
  int64_t wsize = 0;
  for (auto& q : h->host) {
    h->max_nx = std::max<int>(h->max_nx, (int)q.nx);
    h->max_ny = std::max<int>(h->max_ny, (int)q.ny);
    h->max_nkd = std::max<int>(h->max_nkd, (int)q.nkd);
    wsize += wq_pitch(q.nkd, prec == FF_F64 ? 16 : 8) * q.ny;
  }
  const size_t es = prec == FF_F64 ? 16 : 8;
  int st = FF_OK;
  cudaError_t e = cudaMalloc(&h->d_W, 3 * wsize * es);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_Q, 2 * wsize * es);
  if (e != cudaSuccess) st = cuda_status(e, "ff_vort_create: workspace");
  if (st == FF_OK) {
    const char* nog = getenv("FF_NO_GRAPH");
    h->use_graph = !(nog && nog[0] == '1');
    st = rebuild(h, 0, 0, 0, 0);
  }
  if (st != FF_OK) {
    destroy(h);
    return st;
  }
  *out = h;
  return FF_OK;
}

int ff_vort_destroy(ff_vort* h) {
  destroy(h);
  return FF_OK;
}

int ff_vort_step(ff_vort* h, int64_t nsteps, void* stream) {
  FF_CHECK_ARG(h, "ff_vort_step: null handle");
  FF_CHECK_ARG(nsteps >= 0, "ff_vort_step: negative step count");
  auto s = (cudaStream_t)stream;
  const NvtxRange range("ff_vort_step");
  if (!h->use_graph) {
    for (int64_t i = 0; i < nsteps; ++i)
      if (int st = enqueue(h, s)) return st;
    return FF_OK;
  }
  if (!h->exec)
    if (int st = capture(h)) return st;
  for (int64_t i = 0; i < nsteps; ++i) FF_CUDA(cudaGraphLaunch(h->exec, s));
  return FF_OK;
}

int ff_vort_config(const ff_vort* h, int32_t cfg[8]) {
  FF_CHECK_ARG(h && cfg, "ff_vort_config: null argument");
  cfg[0] = h->g.tla;
  cfg[1] = h->g.tlc;
  cfg[2] = h->g.tlr;
  cfg[3] = h->g.reg ? -1 : h->g.radix_variant;  // -1: register-resident power-of-two path
  cfg[4] = h->g.tha;
  cfg[5] = h->g.thb;
  cfg[6] = h->g.thc;
  cfg[7] = h->use_graph ? 1 : 0;
  return FF_OK;
}

int ff_vort_set_config(ff_vort* h, int tla, int tlc, int tlr, int radix_variant) {
  FF_CHECK_ARG(h, "ff_vort_set_config: null handle");
  FF_CHECK_ARG(radix_variant >= 0 && radix_variant <= 2, "ff_vort_set_config: radix variant 0..2");
  FF_CUDA(cudaDeviceSynchronize());
  return rebuild(h, tla, tlc, tlr, radix_variant);
}

int ff_vort_set_split(ff_vort* h, int mode) {
  FF_CHECK_ARG(h, "ff_vort_set_split: null handle");
  FF_CHECK_ARG(mode >= -1 && mode <= 1, "ff_vort_set_split: mode -1 (automatic), 0 or 1");
  FF_CUDA(cudaDeviceSynchronize());
  h->split_mode = mode;
  return rebuild(h, h->g.tla, h->g.tlc, h->g.tlr, h->g.radix_variant);
}

int ff_vort_get_split(const ff_vort* h, int32_t* on) {
  FF_CHECK_ARG(h && on, "ff_vort_get_split: null argument");
  *on = h->g.split_c ? 1 : 0;
  return FF_OK;
}

int ff_vort_autotune(ff_vort* h, int steps_per_trial, void* stream, double* best_ms) {
  FF_CHECK_ARG(h, "ff_vort_autotune: null handle");
  // The trial steps advance the state: callers pass a scratch copy or restore it.
  auto s = (cudaStream_t)stream;
  const int reps = steps_per_trial > 0 ? steps_per_trial : 3;
  const int tls[] = {1, 2, 4, 8};  // lines per CTA of passes A and C, rows per CTA of B
  const int ntl = 4;
  // the register path has one stage schedule; only the generic path varies radix order,
  // and only the register path's unfused pass C can be split by field
  const int nvar = reg_capable(h) ? 1 : 3;
  const bool fused_c = h->prec == FF_F64 ? FuseA<double>::value : FuseA<float>::value;
  const int nsplit = reg_capable(h) && !fused_c ? 2 : 1;
  // the events are destroyed and the caller's split mode is kept on every return path
  struct Guard {
    ff_vort* h;
    int split;
    cudaEvent_t e[2] = {nullptr, nullptr};
    ~Guard() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
      h->split_mode = split;
    }
  } guard{h, h->split_mode};
  FF_CUDA(cudaEventCreate(&guard.e[0]));
  FF_CUDA(cudaEventCreate(&guard.e[1]));
  double best = 1e30;
  int bcfg[5] = {0, 0, 0, 0, guard.split};
  for (int sp = 0; sp < nsplit; ++sp)
    for (int v = 0; v < nvar; ++v)
      for (int ia = 0; ia < ntl; ++ia)
        for (int ic = 0; ic < ntl; ++ic)
          for (int ir = 0; ir < ntl; ++ir) {
            FF_CUDA(cudaStreamSynchronize(s));
            h->split_mode = nsplit > 1 ? sp : guard.split;
            if (int st = rebuild(h, tls[ia], tls[ic], tls[ir], v)) return st;
            // skip configurations the size limits clamped to an already tried one, and
            // split trials whose geometry cannot split
            if (h->g.tla != tls[ia] || h->g.tlc != tls[ic] || h->g.tlr != tls[ir]) continue;
            if (nsplit > 1 && sp == 1 && !h->g.split_c) continue;
            if (int st = ff_vort_step(h, 1, s)) return st;  // warm-up (and graph capture)
            FF_CUDA(cudaEventRecord(guard.e[0], s));
            if (int st = ff_vort_step(h, reps, s)) return st;
            FF_CUDA(cudaEventRecord(guard.e[1], s));
            FF_CUDA(cudaEventSynchronize(guard.e[1]));
            float ms = 0;
            FF_CUDA(cudaEventElapsedTime(&ms, guard.e[0], guard.e[1]));
            const double per = ms / reps;
            if (per < best) {
              best = per;
              bcfg[0] = tls[ia];
              bcfg[1] = tls[ic];
              bcfg[2] = tls[ir];
              bcfg[3] = v;
              bcfg[4] = h->split_mode;
            }
          }
  FF_CUDA(cudaStreamSynchronize(s));
  guard.split = bcfg[4];  // the winner's split mode stays
  h->split_mode = bcfg[4];
  if (int st = rebuild(h, bcfg[0], bcfg[1], bcfg[2], bcfg[3])) return st;
  if (best_ms) *best_ms = best;
  return FF_OK;
}

}  // extern "C"

template <typename T> int profile_t(ff_vort* h, int reps, cudaStream_t s, double ms[3]) {
  if (h->stepper != FF_STEP_ETDRK4 && h->stepper != FF_STEP_RK4) {
    // an LSRK54 stage's epilogue advances the state itself
    set_error("ff_vort_profile: only ETDRK4 and RK4 handles can be profiled without advancing the state");
    return FF_ERR_UNSUPPORTED;
  }
  // every event created is destroyed on every return path, including FF_CUDA's early ones
  struct Events {
    cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
    ~Events() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
    }
  } guard;
  cudaEvent_t* ev = guard.e;
  for (int k = 0; k < 4; ++k) FF_CUDA(cudaEventCreate(&ev[k]));
  double acc[3] = {0, 0, 0};
  int st = FF_OK;
  EpiScalars<T> S{};
  S.c = (T)(h->dt / 2);
  for (int r = 0; r < reps && st == FF_OK; ++r) {
    // pass A on the state, B, then C as the first substep runs it (its epilogue writes
    // only the stepper's intermediate buffers; fused with the next pass A in FP32)
    FF_CUDA(cudaEventRecord(ev[0], s));
    if ((st = launch_a<T>(h, h->d_probs, h->d_work_a, h->nwork_a, h->g.ga, h->d_inputs, s))) break;
    FF_CUDA(cudaEventRecord(ev[1], s));
    if ((st = launch_b<T>(h, h->d_probs, h->d_work_b, h->nwork_b, h->g.gb, s))) break;
    FF_CUDA(cudaEventRecord(ev[2], s));
    {
      const int nw = h->g.reg ? h->nwork_c_kept : h->nwork_c;
      const bool fuse = h->g.reg && FuseA<T>::value;
      const bool split = h->g.split_c;
      st = h->stepper == FF_STEP_RK4
               ? launch_c<T, EPI_RK1>(h, h->d_probs, h->d_work_c, nw, h->g.gc, S, s, fuse, split)
               : launch_c<T, EPI_ETD1>(h, h->d_probs, h->d_work_c, nw, h->g.gc, S, s, fuse, split);
    }
    if (st) break;
    FF_CUDA(cudaEventRecord(ev[3], s));
    FF_CUDA(cudaEventSynchronize(ev[3]));
    for (int k = 0; k < 3; ++k) {
      float t = 0;
      FF_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
      acc[k] += t;
    }
  }
  for (int k = 0; k < 3; ++k) ms[k] = acc[k] / reps;
  return st;
}

extern "C" int ff_vort_profile(ff_vort* h, int reps, void* stream, double ms[3]) {
  FF_CHECK_ARG(h && ms && reps >= 1, "ff_vort_profile: bad argument");
  auto s = (cudaStream_t)stream;
  return h->prec == FF_F64 ? profile_t<double>(h, reps, s, ms) : profile_t<float>(h, reps, s, ms);
}

// a single-problem copy of descriptor `prob` with n1 -> N, its own work lists and the input
// pointer, laid out as [descriptor | work A | work B | work C | input] in `out`
template <typename T>
void calc_stage(const ff_vort* h, int64_t prob, const void* sol, void* N, std::vector<unsigned char>& out, int& nwa,
                int& nwb, int& nwc) {
  const size_t psz = sizeof(VortProb<T>);
  VortProb<T> P;
  memcpy(&P, h->host_desc.data() + psz * prob, psz);
  P.n1 = (cx<T>*)N;
  const Geom& g = h->g;
  const int wa_ = g.reg ? g.tha * 8 / P.ny : g.tla;
  const int wb_ = g.reg ? g.thb * 8 / (P.nx / 2) : g.tlr;
  const int wc_ = g.reg ? g.thc * 8 / P.ny : g.tlc;
  std::vector<WorkItem> wa, wb, wc;
  const int afields = g.reg && AFields<T>::value == 3 ? 1 : 3;
  for (int f = 0; f < afields; ++f)
    for (int t = 0; t < (int)ceil_div(P.nkd, wa_); ++t) wa.push_back({0, t, f, 0});
  for (int t = 0; t < (int)ceil_div(P.ny, wb_); ++t) wb.push_back({0, t, 0, 0});
  for (int t = 0; t < (int)ceil_div(P.nkr, wc_); ++t) wc.push_back({0, t, 0, 0});
  const size_t nw = wa.size() + wb.size() + wc.size();
  out.resize(psz + nw * sizeof(WorkItem) + sizeof(void*));
  unsigned char* hp = out.data();
  memcpy(hp, &P, psz);
  memcpy(hp + psz, wa.data(), wa.size() * sizeof(WorkItem));
  memcpy(hp + psz + wa.size() * sizeof(WorkItem), wb.data(), wb.size() * sizeof(WorkItem));
  memcpy(hp + psz + (wa.size() + wb.size()) * sizeof(WorkItem), wc.data(), wc.size() * sizeof(WorkItem));
  memcpy(hp + psz + nw * sizeof(WorkItem), &sol, sizeof(void*));
  nwa = (int)wa.size();
  nwb = (int)wb.size();
  nwc = (int)wc.size();
}

// the three passes of a staged single-problem calcN! (never split: its own work list)
template <typename T> int calc_launch(const ff_vort* h, const void* dev, int nwa, int nwb, int nwc, cudaStream_t s) {
  const size_t psz = sizeof(VortProb<T>);
  const char* base = (const char*)dev;
  const void* dwa = base + psz;
  const void* dwb = base + psz + nwa * sizeof(WorkItem);
  const void* dwc = base + psz + (nwa + nwb) * sizeof(WorkItem);
  const void* din = base + psz + (nwa + nwb + nwc) * sizeof(WorkItem);
  if (int st = launch_a<T>(h, base, dwa, nwa, nwa, din, s)) return st;
  if (int st = launch_b<T>(h, base, dwb, nwb, nwb, s)) return st;
  return launch_c<T, EPI_N>(h, base, dwc, nwc, nwc, EpiScalars<T>{}, s);
}

template <typename T> int calcN_t(ff_vort* h, int64_t prob, const void* sol, void* N, cudaStream_t s) {
  // staged through a persistent host buffer and copied on the stream
  int nwa, nwb, nwc;
  calc_stage<T>(h, prob, sol, N, h->calc_host, nwa, nwb, nwc);
  const size_t bytes = h->calc_host.size();
  if (bytes > h->calc_cap) {
    // grown at most a few times; the free waits for earlier calls that read it
    if (h->d_calc_prob) cudaFree(h->d_calc_prob);
    h->d_calc_prob = nullptr;
    FF_CUDA(cudaMalloc(&h->d_calc_prob, bytes));
    h->calc_cap = bytes;
  }
  // stream-ordered: kernels of an earlier call on this stream finish first; the host
  // staging buffer may be reused as soon as the call returns (pageable copy)
  FF_CUDA(cudaMemcpyAsync(h->d_calc_prob, h->calc_host.data(), bytes, cudaMemcpyHostToDevice, s));
  return calc_launch<T>(h, h->d_calc_prob, nwa, nwb, nwc, s);
}

template <typename T> int calcN_bind_t(ff_vort* h, int slot, int64_t prob, const void* sol, void* N) {
  std::vector<unsigned char> hp;
  ff_vort::CalcSlot sl;
  calc_stage<T>(h, prob, sol, N, hp, sl.nwa, sl.nwb, sl.nwc);
  if ((size_t)slot >= h->slots.size()) h->slots.resize(slot + 1);
  ff_vort::CalcSlot& cur = h->slots[slot];
  FF_CUDA(cudaDeviceSynchronize());  // a bound slot may be in use by queued launches
  if (cur.d) cudaFree(cur.d);
  cur = ff_vort::CalcSlot{};
  FF_CUDA(cudaMalloc(&sl.d, hp.size()));
  cudaError_t e = cudaMemcpy(sl.d, hp.data(), hp.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(sl.d);
    return cuda_status(e, "ff_vort_calcN_bind: staging");
  }
  sl.gen = h->gen;
  cur = sl;
  return FF_OK;
}

extern "C" int ff_vort_calcN(ff_vort* h, int64_t prob, const void* sol, void* N, void* stream) {
  FF_CHECK_ARG(h && sol && N, "ff_vort_calcN: null argument");
  FF_CHECK_ARG(prob >= 0 && prob < h->nprob, "ff_vort_calcN: problem index out of range");
  auto s = (cudaStream_t)stream;
  return h->prec == FF_F64 ? calcN_t<double>(h, prob, sol, N, s) : calcN_t<float>(h, prob, sol, N, s);
}

extern "C" int ff_vort_calcN_bind(ff_vort* h, int slot, int64_t prob, const void* sol, void* N) {
  FF_CHECK_ARG(h && sol && N, "ff_vort_calcN_bind: null argument");
  FF_CHECK_ARG(slot >= 0 && slot < FF_VORT_CALC_SLOTS, "ff_vort_calcN_bind: slot %d outside 0..%d", slot,
               FF_VORT_CALC_SLOTS - 1);
  FF_CHECK_ARG(prob >= 0 && prob < h->nprob, "ff_vort_calcN_bind: problem index out of range");
  return h->prec == FF_F64 ? calcN_bind_t<double>(h, slot, prob, sol, N) : calcN_bind_t<float>(h, slot, prob, sol, N);
}

extern "C" int ff_vort_calcN_slot(ff_vort* h, int slot, void* stream) {
  FF_CHECK_ARG(h, "ff_vort_calcN_slot: null handle");
  FF_CHECK_ARG(slot >= 0 && slot < (int)h->slots.size() && h->slots[slot].d, "ff_vort_calcN_slot: slot %d is not bound",
               slot);
  const ff_vort::CalcSlot& sl = h->slots[slot];
  FF_CHECK_ARG(sl.gen == h->gen, "ff_vort_calcN_slot: slot %d was bound before the launch geometry changed; bind it "
               "again", slot);
  auto s = (cudaStream_t)stream;
  return h->prec == FF_F64 ? calc_launch<double>(h, sl.d, sl.nwa, sl.nwb, sl.nwc, s)
                           : calc_launch<float>(h, sl.d, sl.nwa, sl.nwb, sl.nwc, s);
}
