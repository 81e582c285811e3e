// Snapshot output: the reference's WriteXDMF (Source/Domain.cpp:1869-2064).
//
// At each output time the reference writes one HDF5 file of float32 datasets
// (Tag and NP int32) in this order: NP, Position (3 per particle), Velocity,
// Acceleration, Tag, Pressure, Density, the three UserOutput properties named
// OutputName[0..2], Mass, h, Sigma and Strain (the six components 00 01 02 11
// 12 22), and an XDMF file (<key>.xmf) that describes them to a viewer. HDF5
// is not linked here: the same datasets, in the same order and types, go back
// to back into one little-endian raw file (<key>.bin), and the .xmf describes
// each as a Format="Binary" DataItem at its byte offset (Seek), with the
// reference's grid, topology and attribute names.
//
// A step's output (psph_output_request) is gathered on the device after the
// step's forces and before its update: the point where Solve writes it
// (Source/Domain.cpp:1773-1788), so positions, velocities, densities and
// pressures are the step's starting state and accelerations the step's own.
// The gather fills a float32 staging buffer laid out like the file; a second
// stream copies it to pinned host memory while the step's update and the
// following steps run, and a host thread writes the two files.
#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <algorithm>

#include "psph_output.cuh"

namespace psph {

namespace {

// Dataset order and widths of the reference's file (Source/Domain.cpp:1933-1972);
// each dataset holds width values per particle.
struct Dataset {
  const char* name;   // nullptr: OutputName[k] of the caller
  int width;
  bool is_int;
};
constexpr int kNumSets = 13;
constexpr Dataset kSets[kNumSets] = {
    {"Position", 3, false}, {"Velocity", 3, false}, {"Acceleration", 3, false}, {"Tag", 1, true},
    {"Pressure", 1, false}, {"Density", 1, false},  {nullptr, 1, false},         {nullptr, 1, false},
    {nullptr, 1, false},    {"Mass", 1, false},     {"h", 1, false},             {"Sigma", 6, false},
    {"Strain", 6, false}};
// staging buffer: set k starts at unit(k) * ncap values (4 bytes each), after
// a 64-byte header whose first int is the particle count; unit(kNumSets) is
// the total width (29 values per particle)
__host__ __device__ constexpr int unit(int k) { return k < 3 ? 3 * k : (k < 11 ? k + 6 : 17 + 6 * (k - 11)); }
constexpr size_t kHeader = 64;

// Rows of the instance's alive particles in Array::DelItems' order (rank by
// original index), as psph_download returns them: flag, then an exclusive
// scan, then per sorted slot the row.
__global__ void out_flag_kernel(DevView v, int lo, int hi, int* __restrict__ flag) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.sc->n || !v.alive[s]) return;
  const int o = cur_persist(v).orig[s];
  if (o >= lo && o < hi) flag[o - lo] = 1;
}

__device__ __forceinline__ void sym6(float* dst, const double* m) {
  dst[0] = (float)m[0];
  dst[1] = (float)m[1];
  dst[2] = (float)m[2];
  dst[3] = (float)m[4];
  dst[4] = (float)m[5];
  dst[5] = (float)m[8];
}

// One sorted slot's values into its row of every dataset (Source/Domain.cpp:1894-1926).
__global__ void out_gather_kernel(DevView v, int lo, int hi, const int* __restrict__ rank, int len, char* stage,
                                  int ncap) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) *reinterpret_cast<int*>(stage) = rank[len];
  if (s >= v.sc->n || !v.alive[s]) return;
  const Persist& P = cur_persist(v);
  const int o = P.orig[s];
  if (o < lo || o >= hi) return;
  const size_t r = (size_t)rank[o - lo], N = (size_t)ncap;
  float* f = reinterpret_cast<float*>(stage + kHeader);
  const double4_32a x = P.X4[s], vel = P.V4[s], a = v.S.A4[s];
  const PClass& C = v.cls[P.cls[s]];
  float* pos = f + unit(0) * N + 3 * r;
  pos[0] = (float)x.x; pos[1] = (float)x.y; pos[2] = (float)x.z;
  float* vo = f + unit(1) * N + 3 * r;
  vo[0] = (float)vel.x; vo[1] = (float)vel.y; vo[2] = (float)vel.z;
  float* ao = f + unit(2) * N + 3 * r;
  ao[0] = (float)a.x; ao[1] = (float)a.y; ao[2] = (float)a.z;
  reinterpret_cast<int*>(f + unit(3) * N)[r] = C.id;
  f[unit(4) * N + r] = (float)vel.w;
  f[unit(5) * N + r] = (float)x.w;
  f[unit(6) * N + r] = 0.f;  // the default UserOutput (OutPut, Source/Domain.cpp:28-33) writes zeros
  f[unit(7) * N + r] = 0.f;
  f[unit(8) * N + r] = 0.f;
  f[unit(9) * N + r] = (float)C.mass;
  f[unit(10) * N + r] = (float)C.h;
  float* sg = f + unit(11) * N + 6 * r;
  float* sn = f + unit(12) * N + 6 * r;
  if (P.sigma) sym6(sg, P.sigma + 9 * (size_t)s);
  else for (int k = 0; k < 6; ++k) sg[k] = 0.f;
  if (P.strain) sym6(sn, P.strain + 9 * (size_t)s);
  else for (int k = 0; k < 6; ++k) sn[k] = 0.f;
}

struct Job {
  std::string key;
  std::string names[3];
  int64_t ncap = 0;
  std::vector<double> props;  // 3 x m host properties (psph_output_write), empty: the zeros gathered
  cudaEvent_t copied = nullptr;
};

bool write_files(const Job& j, const char* host, std::string* err) {
  const int m = *reinterpret_cast<const int*>(host);
  const float* f = reinterpret_cast<const float*>(host + kHeader);
  const size_t N = (size_t)j.ncap;
  const std::string bin = j.key + ".bin";
  FILE* fp = std::fopen(bin.c_str(), "wb");
  if (!fp) {
    *err = "cannot open " + bin + " for writing";
    return false;
  }
  bool ok = std::fwrite(&m, sizeof(int), 1, fp) == 1;  // NP
  size_t seek[kNumSets];
  size_t off = sizeof(int);
  std::vector<float> tmp;
  for (int k = 0; k < kNumSets && ok; ++k) {
    const size_t cnt = (size_t)m * kSets[k].width;
    seek[k] = off;
    const float* src = f + unit(k) * N;
    if (!j.props.empty() && k >= 6 && k <= 8) {  // host properties of psph_output_write
      tmp.resize((size_t)m);
      for (size_t i = 0; i < (size_t)m; ++i) tmp[i] = (float)j.props[(size_t)(k - 6) * m + i];
      src = tmp.data();
    }
    ok = cnt == 0 || std::fwrite(src, sizeof(float), cnt, fp) == cnt;
    off += cnt * sizeof(float);
  }
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) {
    *err = "write to " + bin + " failed";
    return false;
  }
  // the reference's .xmf (Source/Domain.cpp:1986-2062) with Binary data items
  std::string base = bin;
  const size_t slash = base.find_last_of('/');
  if (slash != std::string::npos) base = base.substr(slash + 1);  // relative to the .xmf
  auto item = [&](int k, const char* type) {
    char b[512];
    const int w = kSets[k].width;
    char dims[64];
    if (w == 1) std::snprintf(dims, sizeof dims, "%d", m);
    else std::snprintf(dims, sizeof dims, "%d %d", m, w);
    std::snprintf(b, sizeof b,
                  "       <DataItem Dimensions=\"%s\" NumberType=\"%s\" Precision=\"4\" Format=\"Binary\" "
                  "Endian=\"Little\" Seek=\"%zu\">\n        %s\n       </DataItem>\n",
                  dims, type, seek[k], base.c_str());
    return std::string(b);
  };
  auto attr = [&](int k, const char* name, const char* kind) {
    return std::string("     <Attribute Name=\"") + name + "\" AttributeType=\"" + kind +
           "\" Center=\"Node\">\n" + item(k, kSets[k].is_int ? "Int" : "Float") + "     </Attribute>\n";
  };
  std::string x;
  x += "<?xml version=\"1.0\" ?>\n<!DOCTYPE Xdmf SYSTEM \"Xdmf.dtd\" []>\n<Xdmf Version=\"2.0\">\n <Domain>\n";
  x += "   <Grid Name=\"SPHCenter\" GridType=\"Uniform\">\n";
  x += "     <Topology TopologyType=\"Polyvertex\" NumberOfElements=\"" + std::to_string(m) + "\"/>\n";
  x += "     <Geometry GeometryType=\"XYZ\">\n" + item(0, "Float") + "     </Geometry>\n";
  x += attr(3, "Tag", "Scalar");
  x += attr(0, "Position", "Vector");
  x += attr(1, "Velocity", "Vector");
  x += attr(2, "Acceleration", "Vector");
  x += attr(5, "Density", "Scalar");
  x += attr(4, "Pressure", "Scalar");
  for (int k = 0; k < 3; ++k) x += attr(6 + k, j.names[k].c_str(), "Scalar");
  x += attr(11, "Sigma", "Tensor6");
  x += attr(12, "Strain", "Tensor6");
  x += "   </Grid>\n </Domain>\n</Xdmf>\n";
  const std::string xmf = j.key + ".xmf";
  fp = std::fopen(xmf.c_str(), "w");
  if (!fp) {
    *err = "cannot open " + xmf + " for writing";
    return false;
  }
  ok = std::fwrite(x.data(), 1, x.size(), fp) == x.size();
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) *err = "write to " + xmf + " failed";
  return ok;
}

}  // namespace

struct OutputWriter {
  cudaStream_t copy = nullptr;
  cudaEvent_t gathered = nullptr, copied = nullptr;
  char* d_stage = nullptr;   // device staging buffer
  char* h_stage = nullptr;   // pinned host copy
  size_t bytes = 0;
  int ncap = 0;
  int idx_cap = 0;  // entries of the per-original-index flag / rank arrays
  int* d_flag = nullptr;     // ncap + 1
  int* d_rank = nullptr;     // ncap + 1
  int* d_bs = nullptr;       // scan block sums
  bool copy_pending = false; // the staging buffer's copy has been issued and not waited for by a gather
  // writer thread
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job> jobs;
  bool busy = false, stop = false;
  std::string err;  // first write error, reported by output_flush
};

namespace {
void writer_loop(OutputWriter* w) {
  std::unique_lock<std::mutex> lk(w->mu);
  while (true) {
    w->cv.wait(lk, [w] { return w->stop || !w->jobs.empty(); });
    if (w->jobs.empty()) return;
    Job j = std::move(w->jobs.front());
    w->jobs.pop_front();
    w->busy = true;
    lk.unlock();
    std::string e;
    const cudaError_t ce = cudaEventSynchronize(j.copied);
    if (ce != cudaSuccess) e = std::string("snapshot copy: ") + cudaGetErrorString(ce);
    else write_files(j, w->h_stage, &e);
    lk.lock();
    if (!e.empty() && w->err.empty()) w->err = e;
    w->busy = false;
    w->cv.notify_all();
  }
}

// Buffers for ncap particles whose original indices span len values (more
// than ncap once an in/out-flow boundary has appended particles).
bool ensure(OutputWriter* w, int ncap, int len, std::string* err) {
  auto fail = [&](const char* what, cudaError_t ce) {
    *err = std::string(what) + ": " + cudaGetErrorString(ce);
    return false;
  };
  cudaError_t ce;
  if (!w->copy) {
    if ((ce = cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream", ce);
    if ((ce = cudaEventCreateWithFlags(&w->gathered, cudaEventDisableTiming)) != cudaSuccess ||
        (ce = cudaEventCreateWithFlags(&w->copied, cudaEventDisableTiming)) != cudaSuccess)
      return fail("event", ce);
    w->th = std::thread(writer_loop, w);
  }
  if (!(w->ncap >= ncap && w->d_stage)) {
    const size_t bytes = kHeader + (size_t)unit(kNumSets) * 4 * (size_t)ncap;
    cudaFree(w->d_stage);
    cudaFreeHost(w->h_stage);
    w->d_stage = w->h_stage = nullptr;
    if ((ce = cudaMalloc(&w->d_stage, bytes)) != cudaSuccess) return fail("snapshot staging buffer", ce);
    if ((ce = cudaMallocHost(&w->h_stage, bytes)) != cudaSuccess) return fail("snapshot host buffer", ce);
    w->bytes = bytes;
    w->ncap = ncap;
  }
  const int idx = std::max(ncap, len);
  if (!(w->idx_cap >= idx && w->d_flag)) {
    cudaFree(w->d_flag);
    cudaFree(w->d_rank);
    cudaFree(w->d_bs);
    w->d_flag = w->d_rank = w->d_bs = nullptr;
    if ((ce = cudaMalloc(&w->d_flag, sizeof(int) * ((size_t)idx + 1))) != cudaSuccess ||
        (ce = cudaMalloc(&w->d_rank, sizeof(int) * ((size_t)idx + 1))) != cudaSuccess ||
        (ce = cudaMalloc(&w->d_bs, sizeof(int) * ((size_t)idx / 1024 + 2))) != cudaSuccess)
      return fail("snapshot row buffers", ce);
    w->idx_cap = idx;
  }
  return true;
}
}  // namespace

OutputWriter* output_writer_create() { return new OutputWriter(); }

bool output_flush(OutputWriter* w, std::string* err) {
  if (!w) return true;
  std::unique_lock<std::mutex> lk(w->mu);
  w->cv.wait(lk, [w] { return w->jobs.empty() && !w->busy; });
  if (!w->err.empty()) {
    *err = w->err;
    w->err.clear();
    return false;
  }
  return true;
}

void output_writer_destroy(OutputWriter* w) {
  if (!w) return;
  std::string e;
  output_flush(w, &e);
  {
    std::lock_guard<std::mutex> lk(w->mu);
    w->stop = true;
  }
  w->cv.notify_all();
  if (w->th.joinable()) w->th.join();
  if (w->copy) cudaStreamSynchronize(w->copy);
  cudaFree(w->d_stage);
  cudaFreeHost(w->h_stage);
  cudaFree(w->d_flag);
  cudaFree(w->d_rank);
  cudaFree(w->d_bs);
  if (w->gathered) cudaEventDestroy(w->gathered);
  if (w->copied) cudaEventDestroy(w->copied);
  if (w->copy) cudaStreamDestroy(w->copy);
  delete w;
}

bool output_gather(OutputWriter* w, const DevView& v, int lo, int hi, cudaStream_t st, std::string* err) {
  if (!ensure(w, v.ncap, hi - lo, err)) return false;
  // the staging buffer of the previous output must have left for the host
  if (w->copy_pending) cudaStreamWaitEvent(st, w->copied, 0);
  const int len = hi - lo, nb = (v.ncap + 255) / 256;
  cudaMemsetAsync(w->d_flag, 0, sizeof(int) * ((size_t)len + 1), st);
  out_flag_kernel<<<nb, 256, 0, st>>>(v, lo, hi, w->d_flag);
  launch_exclusive_scan(w->d_flag, w->d_rank, len, w->d_bs, st);
  out_gather_kernel<<<nb, 256, 0, st>>>(v, lo, hi, w->d_rank, len, w->d_stage, v.ncap);
  const cudaError_t ce = cudaEventRecord(w->gathered, st);
  if (ce != cudaSuccess) {
    *err = std::string("snapshot gather: ") + cudaGetErrorString(ce);
    return false;
  }
  return true;
}

bool output_commit(OutputWriter* w, const char* key, const char* const names[3], const double* props, int64_t m,
                   std::string* err) {
  // the pinned buffer is free once the writer has finished the previous job
  {
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv.wait(lk, [w] { return w->jobs.empty() && !w->busy; });
  }
  cudaError_t ce = cudaStreamWaitEvent(w->copy, w->gathered, 0);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(w->h_stage, w->d_stage, w->bytes, cudaMemcpyDeviceToHost, w->copy);
  if (ce == cudaSuccess) ce = cudaEventRecord(w->copied, w->copy);
  if (ce != cudaSuccess) {
    *err = std::string("snapshot copy: ") + cudaGetErrorString(ce);
    return false;
  }
  w->copy_pending = true;
  Job j;
  j.key = key;
  for (int k = 0; k < 3; ++k) j.names[k] = (names && names[k]) ? names[k] : ("Property" + std::to_string(k + 1));
  j.ncap = w->ncap;
  if (props) j.props.assign(props, props + 3 * m);
  j.copied = w->copied;
  {
    std::lock_guard<std::mutex> lk(w->mu);
    w->jobs.push_back(std::move(j));
  }
  w->cv.notify_all();
  return true;
}

}  // namespace psph
