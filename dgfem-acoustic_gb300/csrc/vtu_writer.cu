// Asynchronous VTU snapshot writer (dg_vtu_* in include/dgfem_gb300.h).
//
// The reference writes one VTU per output step from the host state
// (Mesh::writeVTUb, src/Mesh.cpp:1136-1230: points, triangle/tetra cells of
// the corner nodes, per-cell means of p, p/c0^2 and the velocity) through
// VTK's XML writer, whose default is appended data compressed with zlib; the
// whole time loop waits for it. Here:
//   * the cell means are computed on the GPU (the context's stream, so they
//     see the state of every step enqueued before the call) into a device
//     slot, and copied to a pinned host slot on a separate copy stream;
//   * a writer thread waits for the copy, encodes the three cell arrays (zlib
//     blocks compressed by a few threads in parallel, or raw), and writes the
//     file; the mesh part (points, connectivity, offsets, types) is encoded
//     once at creation and reused by every file;
//   * the caller returns as soon as the kernel and the copy are enqueued and
//     continues time stepping; a call blocks only when every slot is still
//     being written (back pressure).
// File layout: VTK XML UnstructuredGrid, header_type UInt64, appended raw
// encoding; compressed arrays use VTK's block layout ([nblocks, block size,
// last block size, compressed sizes...] then the zlib streams).
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "ctx.h"

namespace {

// zlib, loaded at run time (no build-time dependency): compress2 and
// compressBound of the system library
struct Zlib {
  typedef int (*compress2_t)(unsigned char*, unsigned long*, const unsigned char*, unsigned long, int);
  typedef unsigned long (*bound_t)(unsigned long);
  compress2_t compress2 = nullptr;
  bound_t bound = nullptr;
  bool ok = false;
  Zlib() {
    for (const char* name : {"libz.so.1", "libz.so"}) {
      void* h = dlopen(name, RTLD_NOW | RTLD_LOCAL);
      if (!h) continue;
      compress2 = (compress2_t)dlsym(h, "compress2");
      bound = (bound_t)dlsym(h, "compressBound");
      if (compress2 && bound) {
        ok = true;
        return;
      }
    }
  }
};
const Zlib& zlib() {
  static Zlib z;
  return z;
}

constexpr uint64_t kBlock = 32768;  // VTK's default compression block size

void put_u64(std::string& out, uint64_t v) { out.append(reinterpret_cast<const char*>(&v), 8); }

// One appended array: raw ([byte count][bytes]) or zlib blocks.
std::string encode(const void* data, uint64_t bytes, bool compress, int level, int threads) {
  std::string out;
  const unsigned char* src = static_cast<const unsigned char*>(data);
  if (!compress) {
    out.reserve(8 + bytes);
    put_u64(out, bytes);
    out.append(reinterpret_cast<const char*>(src), bytes);
    return out;
  }
  const Zlib& z = zlib();
  const uint64_t nb = bytes == 0 ? 0 : (bytes + kBlock - 1) / kBlock;
  const uint64_t last = bytes == 0 ? 0 : bytes - (nb - 1) * kBlock;
  std::vector<std::vector<unsigned char>> blk(nb);
  std::vector<int> rc(nb, 0);
  auto work = [&](uint64_t b0, uint64_t b1) {
    for (uint64_t b = b0; b < b1; ++b) {
      const uint64_t n = b + 1 == nb ? last : kBlock;
      unsigned long cap = z.bound((unsigned long)n);
      blk[b].resize(cap);
      rc[b] = z.compress2(blk[b].data(), &cap, src + b * kBlock, (unsigned long)n, level);
      blk[b].resize(cap);
    }
  };
  const int nt = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)threads, nb / 4));
  if (nt <= 1) {
    work(0, nb);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(work, nb * t / nt, nb * (t + 1) / nt);
    for (auto& th : pool) th.join();
  }
  for (int r : rc)
    if (r != 0) throw std::runtime_error("zlib compression failed");
  put_u64(out, nb);
  put_u64(out, kBlock);
  put_u64(out, last);
  for (auto& b : blk) put_u64(out, b.size());
  for (auto& b : blk) out.append(reinterpret_cast<const char*>(b.data()), b.size());
  return out;
}

__global__ void k_vtu_cells(const void* u, int fp32, const int* perm, int64_t E, int np, int nv, int64_t stride,
                            double c0sq, double* out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  double p = 0.0, rho = 0.0, v[3] = {0.0, 0.0, 0.0};
  for (int n = 0; n < np; ++n) {
    const int64_t g = e * np + perm[n];
    const double pv = fp32 ? (double)((const float*)u)[g] : ((const double*)u)[g];
    p += pv;
    rho += pv / c0sq;
    for (int d = 0; d < nv - 1; ++d)
      v[d] += fp32 ? (double)((const float*)u)[(1 + d) * stride + g] : ((const double*)u)[(1 + d) * stride + g];
  }
  // VTU layout: pressure [E], density [E], velocity [E][3]
  out[e] = p / np;
  out[E + e] = rho / np;
  for (int d = 0; d < 3; ++d) out[2 * E + 3 * e + d] = v[d] / np;
}

}  // namespace

struct dg_vtu_writer {
  dg_ctx* c = nullptr;
  int64_t E = 0, npts = 0;
  bool compress = false;
  int level = 1, threads = 4;
  std::string mesh_blob;   // encoded points, connectivity, offsets, types (shared by every file)
  uint64_t mesh_off[4] = {0, 0, 0, 0};
  struct Slot {
    double* d = nullptr;
    double* h = nullptr;
    cudaEvent_t computed = nullptr, copied = nullptr;
    bool busy = false;
  };
  std::vector<Slot> slots;
  cudaStream_t copy = nullptr;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv_job, cv_free;
  std::deque<std::pair<int, std::string>> jobs;
  bool stop = false;
  std::string err, first_err;
  int64_t written = 0;
};

namespace {

int vfail(dg_vtu_writer* w, int code, const std::string& m) {
  if (w) w->err = m;
  return code;
}

void write_file(dg_vtu_writer* w, const double* cells, const std::string& path) {
  const int64_t E = w->E;
  const std::string p = encode(cells, (uint64_t)E * 8, w->compress, w->level, w->threads);
  const std::string r = encode(cells + E, (uint64_t)E * 8, w->compress, w->level, w->threads);
  const std::string v = encode(cells + 2 * E, (uint64_t)E * 24, w->compress, w->level, w->threads);
  const uint64_t o4 = w->mesh_blob.size(), o5 = o4 + p.size(), o6 = o5 + r.size();
  char buf[4096];
  std::string xml;
  std::snprintf(buf, sizeof(buf),
                "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" "
                "byte_order=\"LittleEndian\" header_type=\"UInt64\"%s>\n  <UnstructuredGrid>\n"
                "    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n",
                w->compress ? " compressor=\"vtkZLibDataCompressor\"" : "", (long long)w->npts, (long long)E);
  xml += buf;
  std::snprintf(buf, sizeof(buf),
                "      <Points>\n        <DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"appended\" "
                "offset=\"%llu\"/>\n      </Points>\n      <Cells>\n"
                "        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"appended\" offset=\"%llu\"/>\n"
                "        <DataArray type=\"Int64\" Name=\"offsets\" format=\"appended\" offset=\"%llu\"/>\n"
                "        <DataArray type=\"UInt8\" Name=\"types\" format=\"appended\" offset=\"%llu\"/>\n      </Cells>\n",
                (unsigned long long)w->mesh_off[0], (unsigned long long)w->mesh_off[1],
                (unsigned long long)w->mesh_off[2], (unsigned long long)w->mesh_off[3]);
  xml += buf;
  std::snprintf(buf, sizeof(buf),
                "      <CellData>\n        <DataArray type=\"Float64\" Name=\"Pressure [Pa]\" format=\"appended\" "
                "offset=\"%llu\"/>\n        <DataArray type=\"Float64\" Name=\"Density [kg/m³]\" format=\"appended\" "
                "offset=\"%llu\"/>\n        <DataArray type=\"Float64\" Name=\"Velocity [m/s]\" NumberOfComponents=\"3\" "
                "format=\"appended\" offset=\"%llu\"/>\n      </CellData>\n"
                "    </Piece>\n  </UnstructuredGrid>\n  <AppendedData encoding=\"raw\">\n   _",
                (unsigned long long)o4, (unsigned long long)o5, (unsigned long long)o6);
  xml += buf;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  bool ok = std::fwrite(xml.data(), 1, xml.size(), f) == xml.size();
  ok = ok && std::fwrite(w->mesh_blob.data(), 1, w->mesh_blob.size(), f) == w->mesh_blob.size();
  for (const std::string* s : {&p, &r, &v}) ok = ok && std::fwrite(s->data(), 1, s->size(), f) == s->size();
  const char* tail = "\n  </AppendedData>\n</VTKFile>\n";
  ok = ok && std::fputs(tail, f) >= 0;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) throw std::runtime_error("write error on " + path);
}

void worker_main(dg_vtu_writer* w) {
  for (;;) {
    std::pair<int, std::string> job;
    {
      std::unique_lock<std::mutex> lk(w->mu);
      w->cv_job.wait(lk, [&] { return w->stop || !w->jobs.empty(); });
      if (w->jobs.empty()) return;  // stop with nothing left
      job = w->jobs.front();
      w->jobs.pop_front();
    }
    dg_vtu_writer::Slot& s = w->slots[job.first];
    std::string e;
    cudaError_t ce = cudaEventSynchronize(s.copied);
    if (ce != cudaSuccess) {
      e = std::string("CUDA (snapshot copy): ") + cudaGetErrorString(ce);
    } else {
      try {
        write_file(w, s.h, job.second);
      } catch (const std::exception& ex) {
        e = ex.what();
      }
    }
    {
      std::lock_guard<std::mutex> lk(w->mu);
      if (!e.empty() && w->first_err.empty()) w->first_err = e;
      s.busy = false;
      if (e.empty()) ++w->written;
    }
    w->cv_free.notify_all();
  }
}

}  // namespace

extern "C" {

int dg_vtu_writer_create(dg_ctx* c, int64_t n_points, const double* points, const int64_t* cells, int compression,
                         int n_slots, dg_vtu_writer** out) {
  if (!out) return DG_ERR_ARG;
  *out = nullptr;
  if (!c || n_points <= 0 || !points || !cells || compression < -1 || compression > 1 || n_slots < 0 || n_slots > 64)
    return DG_ERR_ARG;
  auto* w = new dg_vtu_writer;
  w->c = c;
  w->E = c->E;
  w->npts = n_points;
  const bool zok = zlib().ok;
  if (compression == 1 && !zok) {
    delete w;
    return DG_ERR_ARG;  // zlib requested but the system library is not there
  }
  w->compress = compression == 1 || (compression == -1 && zok);
  w->threads = (int)std::max(1u, std::min(8u, std::thread::hardware_concurrency() / 2));
  const int nc = c->dim + 1;
  for (int64_t k = 0; k < c->E * nc; ++k)
    if (cells[k] < 0 || cells[k] >= n_points) {
      delete w;
      return DG_ERR_ARG;
    }
  // mesh part, encoded once
  std::vector<int64_t> offs(c->E);
  std::vector<uint8_t> types(c->E, c->dim == 3 ? 10 : c->dim == 2 ? 5 : 3);  // VTK_TETRA, VTK_TRIANGLE, VTK_LINE
  for (int64_t e = 0; e < c->E; ++e) offs[e] = (e + 1) * nc;
  try {
    const std::string a = encode(points, (uint64_t)n_points * 24, w->compress, w->level, w->threads);
    const std::string b = encode(cells, (uint64_t)c->E * nc * 8, w->compress, w->level, w->threads);
    const std::string d = encode(offs.data(), (uint64_t)c->E * 8, w->compress, w->level, w->threads);
    const std::string t = encode(types.data(), (uint64_t)c->E, w->compress, w->level, w->threads);
    w->mesh_off[0] = 0, w->mesh_off[1] = a.size(), w->mesh_off[2] = a.size() + b.size();
    w->mesh_off[3] = w->mesh_off[2] + d.size();
    w->mesh_blob = a + b + d + t;
  } catch (const std::exception&) {
    delete w;
    return DG_ERR_ARG;
  }
  const int ns = n_slots == 0 ? 3 : n_slots;
  w->slots.resize(ns);
  cudaError_t e = cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking);
  for (auto& s : w->slots) {
    if (e == cudaSuccess) e = cudaMalloc(&s.d, (size_t)c->E * 5 * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&s.h, (size_t)c->E * 5 * sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.computed, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.copied, cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    for (auto& s : w->slots) {
      if (s.d) cudaFree(s.d);
      if (s.h) cudaFreeHost(s.h);
      if (s.computed) cudaEventDestroy(s.computed);
      if (s.copied) cudaEventDestroy(s.copied);
    }
    if (w->copy) cudaStreamDestroy(w->copy);
    delete w;
    return DG_ERR_CUDA;
  }
  w->worker = std::thread(worker_main, w);
  *out = w;
  return DG_OK;
}

int dg_vtu_write_async(dg_vtu_writer* w, const char* path) {
  if (!w || !path || !*path) return DG_ERR_ARG;
  dg_ctx* c = w->c;
  int k = -1;
  {
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv_free.wait(lk, [&] {
      for (size_t i = 0; i < w->slots.size(); ++i)
        if (!w->slots[i].busy) return true;
      return false;
    });
    for (size_t i = 0; i < w->slots.size() && k < 0; ++i)
      if (!w->slots[i].busy) k = (int)i;
    w->slots[k].busy = true;
  }
  dg_vtu_writer::Slot& s = w->slots[k];
  auto undo = [&](cudaError_t e) {
    std::lock_guard<std::mutex> lk(w->mu);
    s.busy = false;
    w->cv_free.notify_all();
    return vfail(w, DG_ERR_CUDA, std::string("CUDA (snapshot): ") + cudaGetErrorString(e));
  };
  const int64_t E = c->E;
  k_vtu_cells<<<(unsigned)((E + 127) / 128), 128, 0, c->stream>>>(c->u, c->prec == DG_FP32 ? 1 : 0, c->d_perm, E,
                                                                  c->np, c->nv, c->Epad * c->np, c->c0sq, s.d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventRecord(s.computed, c->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(w->copy, s.computed, 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s.h, s.d, (size_t)E * 5 * sizeof(double), cudaMemcpyDeviceToHost, w->copy);
  if (e == cudaSuccess) e = cudaEventRecord(s.copied, w->copy);
  if (e != cudaSuccess) return undo(e);
  {
    std::lock_guard<std::mutex> lk(w->mu);
    w->jobs.emplace_back(k, std::string(path));
  }
  w->cv_job.notify_one();
  return DG_OK;
}

int dg_vtu_writer_flush(dg_vtu_writer* w) {
  if (!w) return DG_ERR_ARG;
  std::unique_lock<std::mutex> lk(w->mu);
  w->cv_free.wait(lk, [&] {
    if (!w->jobs.empty()) return false;
    for (auto& s : w->slots)
      if (s.busy) return false;
    return true;
  });
  if (!w->first_err.empty()) {
    w->err = w->first_err;
    w->first_err.clear();
    return DG_ERR_ARG;
  }
  return DG_OK;
}

int dg_vtu_writer_destroy(dg_vtu_writer* w) {
  if (!w) return DG_OK;
  int rc = dg_vtu_writer_flush(w);
  {
    std::lock_guard<std::mutex> lk(w->mu);
    w->stop = true;
  }
  w->cv_job.notify_all();
  if (w->worker.joinable()) w->worker.join();
  for (auto& s : w->slots) {
    cudaFree(s.d);
    cudaFreeHost(s.h);
    cudaEventDestroy(s.computed);
    cudaEventDestroy(s.copied);
  }
  cudaStreamDestroy(w->copy);
  delete w;
  return rc;
}

const char* dg_vtu_writer_last_error(const dg_vtu_writer* w) { return w ? w->err.c_str() : ""; }

int dg_vtu_writer_stats(const dg_vtu_writer* w, int64_t* files_written, int* compressed) {
  if (!w) return DG_ERR_ARG;
  auto* mw = const_cast<dg_vtu_writer*>(w);
  std::lock_guard<std::mutex> lk(mw->mu);
  if (files_written) *files_written = w->written;
  if (compressed) *compressed = w->compress ? 1 : 0;
  return DG_OK;
}

}  // extern "C"
