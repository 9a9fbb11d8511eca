// Output writers of the drop-in driver and the WAV reader:
//   * results/result<step>.vtu (src/Mesh.cpp:1136-1230): points = all mesh
//     nodes at index tag-1, linear cells from the first dim+1 element nodes,
//     cell data "Pressure [Pa]", "Density [kg/m³]", "Velocity [m/s]"; written
//     as VTK XML with raw appended binary data;
//   * results.pvd (src/Mesh.cpp:1232-1253), replaying the time loop;
//   * observer WAV files, 16-bit mono PCM, value*32767 truncated, sample rate
//     (uint32)(1/dt) (src/utils.cpp:179-211, src/wave/file.cc:314-325);
//   * observer spectra _fft.txt / _psd.txt (src/utils.cpp:260-296,
//     src/fft.cpp:96-100, :146-271) with an in-house radix-2 FFT in place of
//     FFTW (the sizes are powers of two);
//   * WAV reading for file sources (src/wave/file.cc:246-290 scaling).
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dgfem_host.h"
#include "config.h"
#include "host_common.h"
#include "mshio.h"

namespace dgout {

namespace {
[[noreturn]] void fail(const std::string& m) { throw std::runtime_error(m); }

void put_u32(std::vector<unsigned char>& b, uint32_t v) {
  for (int i = 0; i < 4; ++i) b.push_back((unsigned char)(v >> (8 * i)));
}
void put_u16(std::vector<unsigned char>& b, uint16_t v) {
  b.push_back((unsigned char)v), b.push_back((unsigned char)(v >> 8));
}
uint32_t get_u32(const unsigned char* p) { return p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24); }
uint16_t get_u16(const unsigned char* p) { return (uint16_t)(p[0] | (p[1] << 8)); }
}  // namespace

void write_wav(const std::string& path, const float* s, int64_t n, uint32_t rate) {
  std::vector<unsigned char> b;
  const uint16_t bits = 16, ch = 1;
  uint32_t data_bytes = (uint32_t)(n * 2);
  b.insert(b.end(), {'R', 'I', 'F', 'F'});
  put_u32(b, 36 + data_bytes);
  b.insert(b.end(), {'W', 'A', 'V', 'E', 'f', 'm', 't', ' '});
  put_u32(b, 16);
  put_u16(b, 1);
  put_u16(b, ch);
  put_u32(b, rate);
  put_u32(b, rate * ch * bits / 8);
  put_u16(b, ch * bits / 8);
  put_u16(b, bits);
  b.insert(b.end(), {'d', 'a', 't', 'a'});
  put_u32(b, data_bytes);
  for (int64_t i = 0; i < n; ++i) {
    float f = s[i] * (float)std::numeric_limits<int16_t>::max();
    // float -> int16 by truncation; out-of-range values wrap like an
    // int32 conversion truncated to 16 bits
    int32_t w = std::isfinite(f) && std::fabs(f) < 2147483520.0f ? (int32_t)f : 0;
    int16_t v = (int16_t)(uint16_t)(uint32_t)w;
    put_u16(b, (uint16_t)v);
  }
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) fail("cannot write " + path);
  std::fwrite(b.data(), 1, b.size(), fp);
  std::fclose(fp);
}

void read_wav(const std::string& path, std::vector<float>& out, uint32_t& rate) {
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open()) fail("cannot open WAV file " + path);
  std::vector<unsigned char> b((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  if (b.size() < 12 || std::memcmp(b.data(), "RIFF", 4) || std::memcmp(b.data() + 8, "WAVE", 4))
    fail("not a RIFF/WAVE file: " + path);
  size_t pos = 12;
  uint16_t bits = 0, ch = 1;
  rate = 0;
  const unsigned char* data = nullptr;
  uint32_t data_bytes = 0;
  while (pos + 8 <= b.size()) {
    uint32_t sz = get_u32(&b[pos + 4]);
    if (!std::memcmp(&b[pos], "fmt ", 4) && pos + 8 + 16 <= b.size()) {
      ch = get_u16(&b[pos + 10]);
      rate = get_u32(&b[pos + 12]);
      bits = get_u16(&b[pos + 22]);
    } else if (!std::memcmp(&b[pos], "data", 4)) {
      data = &b[pos + 8];
      data_bytes = (uint32_t)std::min<size_t>(sz, b.size() - pos - 8);
      break;
    }
    pos += 8 + sz + (sz & 1);
  }
  if (!data || bits == 0) fail("WAV file without fmt/data chunk: " + path);
  (void)ch;
  size_t bps = bits / 8, n = data_bytes / bps;
  out.resize(n);
  for (size_t i = 0; i < n; ++i) {
    const unsigned char* q = data + i * bps;
    if (bits == 8) out[i] = (float)(int8_t)q[0] / std::numeric_limits<int8_t>::max();
    else if (bits == 16) out[i] = (float)(int16_t)get_u16(q) / std::numeric_limits<int16_t>::max();
    else if (bits == 24) {
      int v = (q[2] & 0x80) ? (int)((0xffu << 24) | (q[2] << 16) | (q[1] << 8) | q[0]) : (q[2] << 16) | (q[1] << 8) | q[0];
      out[i] = (float)v / 8388607;
    } else if (bits == 32) out[i] = (float)(int32_t)get_u32(q) / std::numeric_limits<int32_t>::max();
    else fail("unsupported WAV sample size");
  }
}

// In-place iterative radix-2 forward DFT (X_k = sum x_n e^{-2 pi i k n / N}).
void fft(std::vector<std::complex<double>>& a) {
  size_t n = a.size();
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    double ang = -2.0 * M_PI / (double)len;
    for (size_t i = 0; i < n; i += len)
      for (size_t k = 0; k < len / 2; ++k) {
        std::complex<double> w(std::cos(ang * k), std::sin(ang * k));
        std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
      }
  }
}

// src/fft.cpp:96-100
size_t nearest_lower_pow2(size_t number) {
  size_t n = (size_t)std::floor(std::log((double)number) / std::log(2.0));
  return (size_t)std::pow(2, (double)n);
}

// Rows of the two spectrum files for a pressure trace.
void spectra(const float* V, int64_t count, double dt, int64_t* nb_out, std::vector<double>& fftrows,
             std::vector<double>& psdrows) {
  if (count < 2) fail("spectra need at least two samples");
  size_t nb = nearest_lower_pow2((size_t)count);
  std::vector<double> tcol(nb), pcol(nb);
  double sum = 0.0;
  for (size_t i = 0; i < nb; ++i) {
    tcol[i] = i * dt;
    pcol[i] = V[i];
    sum += pcol[i];
  }
  sum /= (double)nb;
  for (auto& v : pcol) v = v - sum;
  std::vector<std::complex<double>> y(nb);
  for (size_t i = 0; i < nb; ++i) y[i] = {pcol[i], 0.0};
  fft(y);
  // amplitude spectrum (FFTW_spec)
  double periods = tcol[nb - 1] - tcol[0];
  fftrows.assign((nb / 2) * 5, 0.0);
  for (size_t i = 0; i < nb / 2; ++i) {
    double norm = 2.0 * std::sqrt(std::pow(y[i].real(), 2) + std::pow(y[i].imag(), 2)) / nb;
    fftrows[i * 5 + 0] = i / periods;
    fftrows[i * 5 + 1] = norm;
    fftrows[i * 5 + 2] = y[i].real();
    fftrows[i * 5 + 3] = y[i].imag();
    fftrows[i * 5 + 4] = 20.0 * std::log10(norm / 2.0E-5);
  }
  // one-sided PSD (PSD_spec)
  double sampleRate = 1. / (tcol[nb - 1] - tcol[0]);
  const double nf = (1. / double(nb * nb)) * (1. / sampleRate);
  psdrows.assign((nb / 2 + 1) * 3, 0.0);
  psdrows[0] = 0.0;
  psdrows[1] = (std::pow(y[0].real(), 2) + std::pow(y[0].imag(), 2)) * nf;
  psdrows[2] = 10.0 * std::log10(psdrows[1] / std::pow(2.0E-5, 2));
  for (size_t i = 1; i < nb / 2 + 1; ++i) {
    double P = std::pow(y[i].real(), 2) + std::pow(y[i].imag(), 2);
    psdrows[i * 3 + 0] = i * sampleRate;
    psdrows[i * 3 + 1] = 2.0 * P * nf;
    psdrows[i * 3 + 2] = 10.0 * std::log10(psdrows[i * 3 + 1] / std::pow(2.0E-5, 2));
  }
  if (nb % 2 == 0) {
    psdrows[(nb / 2) * 3 + 1] *= 0.5;
    psdrows[(nb / 2) * 3 + 2] = 10.0 * std::log10(psdrows[(nb / 2) * 3 + 1] / std::pow(2.0E-5, 2));
  }
  *nb_out = (int64_t)nb;
}

void write_spectra(const std::string& prefix, const float* V, int64_t count, double dt) {
  int64_t nb;
  std::vector<double> f, p;
  spectra(V, count, dt, &nb, f, p);
  FILE* a = std::fopen((prefix + "_fft.txt").c_str(), "w");
  if (!a) fail("cannot write " + prefix + "_fft.txt");
  std::fprintf(a, "Frequency Norm Real Imag SPL\n");
  for (int64_t i = 1; i < nb / 2; ++i) {
    for (int j = 0; j < 5; ++j) std::fprintf(a, "%g ", f[i * 5 + j]);
    std::fprintf(a, "\n");
  }
  std::fclose(a);
  FILE* b = std::fopen((prefix + "_psd.txt").c_str(), "w");
  if (!b) fail("cannot write " + prefix + "_psd.txt");
  std::fprintf(b, "Frequency Norm PSD\n");
  for (int64_t i = 1; i < nb / 2 + 1; ++i) {
    for (int j = 0; j < 3; ++j) std::fprintf(b, "%g ", p[i * 3 + j]);
    std::fprintf(b, "\n");
  }
  std::fclose(b);
}

void write_vtu(const std::string& path, int dim, const std::vector<int64_t>& node_tags, const std::vector<double>& xyz,
               int nodes_per_elem, const std::vector<int64_t>& elem_nodes, const double* cp, const double* crho,
               const double* cv) {
  int64_t N = (int64_t)node_tags.size(), E = (int64_t)elem_nodes.size() / nodes_per_elem;
  int64_t maxtag = 0;
  for (auto t : node_tags) maxtag = std::max(maxtag, t);
  // points at index tag-1
  std::vector<double> pts(3 * maxtag, 0.0);
  for (int64_t i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) pts[3 * (node_tags[i] - 1) + d] = xyz[3 * i + d];
  int nc = dim + 1;
  std::vector<int64_t> conn(E * nc), offs(E);
  std::vector<uint8_t> types(E, dim == 3 ? 10 : dim == 2 ? 5 : 3);  // VTK_TETRA, VTK_TRIANGLE, VTK_LINE
  for (int64_t e = 0; e < E; ++e) {
    for (int k = 0; k < nc; ++k) conn[e * nc + k] = node_tags[elem_nodes[e * nodes_per_elem + k]] - 1;
    offs[e] = (e + 1) * nc;
  }
  std::vector<double> vel(3 * E);
  for (int64_t i = 0; i < 3 * E; ++i) vel[i] = cv[i];
  struct Arr {
    const void* p;
    uint64_t bytes;
  };
  std::vector<Arr> arrs = {{pts.data(), pts.size() * 8},   {conn.data(), conn.size() * 8}, {offs.data(), offs.size() * 8},
                           {types.data(), types.size()},   {cp, (uint64_t)E * 8},          {crho, (uint64_t)E * 8},
                           {vel.data(), vel.size() * 8}};
  std::vector<uint64_t> off(arrs.size());
  uint64_t acc = 0;
  for (size_t i = 0; i < arrs.size(); ++i) off[i] = acc, acc += 8 + arrs[i].bytes;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) fail("cannot write " + path);
  std::fprintf(f,
               "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" "
               "header_type=\"UInt64\">\n  <UnstructuredGrid>\n    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n",
               (long long)maxtag, (long long)E);
  std::fprintf(f,
               "      <Points>\n        <DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"appended\" "
               "offset=\"%llu\"/>\n      </Points>\n",
               (unsigned long long)off[0]);
  std::fprintf(f,
               "      <Cells>\n        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"appended\" offset=\"%llu\"/>\n"
               "        <DataArray type=\"Int64\" Name=\"offsets\" format=\"appended\" offset=\"%llu\"/>\n"
               "        <DataArray type=\"UInt8\" Name=\"types\" format=\"appended\" offset=\"%llu\"/>\n      </Cells>\n",
               (unsigned long long)off[1], (unsigned long long)off[2], (unsigned long long)off[3]);
  std::fprintf(f,
               "      <CellData>\n        <DataArray type=\"Float64\" Name=\"Pressure [Pa]\" format=\"appended\" "
               "offset=\"%llu\"/>\n        <DataArray type=\"Float64\" Name=\"Density [kg/m³]\" format=\"appended\" "
               "offset=\"%llu\"/>\n        <DataArray type=\"Float64\" Name=\"Velocity [m/s]\" NumberOfComponents=\"3\" "
               "format=\"appended\" offset=\"%llu\"/>\n      </CellData>\n",
               (unsigned long long)off[4], (unsigned long long)off[5], (unsigned long long)off[6]);
  std::fprintf(f, "    </Piece>\n  </UnstructuredGrid>\n  <AppendedData encoding=\"raw\">\n   _");
  for (auto& a : arrs) {
    uint64_t n = a.bytes;
    std::fwrite(&n, 8, 1, f);
    if (n) std::fwrite(a.p, 1, n, f);
  }
  std::fprintf(f, "\n  </AppendedData>\n</VTKFile>\n");
  std::fclose(f);
}

// src/Mesh.cpp:1232-1253
void write_pvd(const std::string& path, double t_start, double t_end, double dt, double t_rate) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) fail("cannot write " + path);
  std::fprintf(f, "<VTKFile type=\"Collection\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n");
  std::fprintf(f, "  <Collection>\n");
  for (double t = t_start, step = 0, tDisplay = 0; t <= t_end; t += dt, tDisplay += dt, ++step) {
    if (tDisplay >= t_rate || step == 0) {
      tDisplay = 0;
      std::fprintf(f, "    <DataSet timestep=\"%g\" part=\"0\" file=\"results/result%d.vtu\"/>\n", t, (int)step);
    }
    if (!(dt > 0)) break;
  }
  std::fprintf(f, "  </Collection>\n</VTKFile>\n");
  std::fclose(f);
}

}  // namespace dgout

namespace dgcfg {
std::vector<double> read_wav_table(const std::string& path) {
  std::vector<float> V;
  uint32_t rate = 0;
  dgout::read_wav(path, V, rate);
  if (rate == 0) throw std::runtime_error("WAV sample rate is zero: " + path);
  std::vector<double> tab;
  double step = 1.0 / rate, time = 0.0;
  for (float v : V) {
    tab.push_back(time);
    tab.push_back(v);
    time += step;
  }
  return tab;
}
}  // namespace dgcfg
