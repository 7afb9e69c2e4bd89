// Restart files of WriteRestart / ReadRestart (INIT/Restart_Mod.f90:14-82).
//
// The reference writes one file per MPI rank, 'RESTART/<grid file up to the
// dot of ".grid"><rank>', as a Fortran unformatted sequential file (gfortran,
// INTEGER = 4 bytes, REAL(RealKind) = 8 bytes, native little endian):
//   record 1: Time            (REAL 8)
//   record 2: GMVStep         (INTEGER 4)
//   record 3: OutputTime      (REAL 8)
//   per local block ib:
//     one record per component ic: Vec(ib)%Vec(ic)%c(ix0:ix1+1,iy0:iy1+1,iz0:iz1+1,1:nFrac)
//     one record:                  uF(ix0:ix1,..), vF(..), wF(..) back to back
// A record is one or more subrecords, each [marker][bytes][marker] with
// 4-byte markers holding the subrecord's byte count; a record longer than the
// maximum subrecord length (gfortran: 2 GiB - 9 bytes) is split, the leading
// marker is negative when another subrecord follows, the trailing one is
// negative when one preceded it.
//
// The library's padded cell layout and face layout are exactly the
// reference's array extents in column-major order, so each record is one
// contiguous array.  Device arrays move through two pinned staging buffers on
// a private stream: the copy of one chunk overlaps the file transfer of the
// other.  Host arrays go to the file directly.
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

namespace {

constexpr long long kGfortranMaxSubrecord = 2147483639LL;
long long g_max_subrecord = kGfortranMaxSubrecord;
constexpr size_t kChunk = size_t(32) << 20;

struct Seg {
  char* p;       // start of the array (device or host)
  size_t bytes;  // its size
  bool dev;
};

int io_fail(const std::string& msg) {
  asam::set_last_error(msg.c_str(), __FILE__, __LINE__);
  return ASAM_IO_ERROR;
}

int cuda_fail(cudaError_t e) {
  asam::set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
  return ASAM_CUDA_ERROR;
}
#define RCU(expr)                          \
  do {                                     \
    cudaError_t e_ = (expr);               \
    if (e_ != cudaSuccess) return cuda_fail(e_); \
  } while (0)

int arg_fail(const std::string& msg) {
  asam::set_last_error(msg.c_str(), __FILE__, __LINE__);
  return ASAM_BAD_ARG;
}

bool on_device(const void* p) { return asam::device_array(p); }

struct Stage {
  char* pin[2] = {nullptr, nullptr};
  cudaStream_t st = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool ready = false;
  int init() {
    if (ready) return ASAM_OK;
    for (int b = 0; b < 2; ++b) {
      RCU(cudaHostAlloc((void**)&pin[b], kChunk, cudaHostAllocDefault));
      RCU(cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming));
    }
    RCU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    ready = true;
    return ASAM_OK;
  }
  ~Stage() {
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
    for (int b = 0; b < 2; ++b) {
      if (ev[b]) cudaEventDestroy(ev[b]);
      if (pin[b]) cudaFreeHost(pin[b]);
    }
  }
};

// A piece of a subrecord's payload: bytes [off, off+len) of segment s.
struct Piece {
  int s;
  size_t off, len;
};

// Cut payload bytes [from, from+len) of a record (its segments back to back)
// into pieces that stay inside one segment and one staging chunk.
void cut(const std::vector<Seg>& segs, size_t from, size_t len, std::vector<Piece>& out) {
  out.clear();
  size_t base = 0;
  for (int s = 0; s < (int)segs.size() && len > 0; ++s) {
    size_t b = segs[s].bytes;
    if (from < base + b) {
      size_t o = from - base;
      size_t take = std::min(b - o, len);
      for (size_t q = 0; q < take; q += kChunk) out.push_back(Piece{s, o + q, std::min(kChunk, take - q)});
      from += take;
      len -= take;
    }
    base += b;
  }
}

bool put_marker(FILE* f, long long v) {
  int32_t m = (int32_t)v;
  return fwrite(&m, 4, 1, f) == 1;
}

bool get_marker(FILE* f, int32_t* m) { return fread(m, 4, 1, f) == 1; }

// Write one record (segments back to back), split into subrecords.
int write_record(FILE* f, const std::vector<Seg>& segs, Stage& sg, const char* what) {
  size_t total = 0;
  for (auto& s : segs) total += s.bytes;
  const size_t maxsub = (size_t)g_max_subrecord;
  const size_t nsub = total == 0 ? 1 : (total + maxsub - 1) / maxsub;
  std::vector<Piece> pcs;
  for (size_t k = 0; k < nsub; ++k) {
    const size_t from = k * maxsub;
    const size_t len = std::min(maxsub, total - from);
    const long long lead = (k + 1 < nsub) ? -(long long)len : (long long)len;
    const long long tail = (k > 0) ? -(long long)len : (long long)len;
    if (!put_marker(f, lead)) return io_fail(std::string("restart write failed at ") + what + ": " + strerror(errno));
    cut(segs, from, len, pcs);
    auto issue = [&](size_t i) -> cudaError_t {
      const Piece& p = pcs[i];
      if (!segs[p.s].dev) return cudaSuccess;
      cudaError_t e = cudaMemcpyAsync(sg.pin[i & 1], segs[p.s].p + p.off, p.len, cudaMemcpyDeviceToHost, sg.st);
      return e != cudaSuccess ? e : cudaEventRecord(sg.ev[i & 1], sg.st);
    };
    if (!pcs.empty()) RCU(issue(0));
    for (size_t i = 0; i < pcs.size(); ++i) {
      if (i + 1 < pcs.size()) RCU(issue(i + 1));
      const Piece& p = pcs[i];
      const char* src = segs[p.s].p + p.off;
      if (segs[p.s].dev) {
        RCU(cudaEventSynchronize(sg.ev[i & 1]));
        src = sg.pin[i & 1];
      }
      if (fwrite(src, 1, p.len, f) != p.len)
        return io_fail(std::string("restart write failed at ") + what + ": " + strerror(errno));
    }
    if (!put_marker(f, tail)) return io_fail(std::string("restart write failed at ") + what + ": " + strerror(errno));
  }
  return ASAM_OK;
}

// Read one record into segments; its length must be the segments' total.
int read_record(FILE* f, const std::vector<Seg>& segs, Stage& sg, const char* what) {
  size_t total = 0;
  for (auto& s : segs) total += s.bytes;
  size_t got = 0;
  bool first = true;
  std::vector<Piece> pcs;
  for (;;) {
    int32_t lead, tail;
    if (!get_marker(f, &lead)) return io_fail(std::string("restart file ends before ") + what);
    const size_t len = (size_t)(lead < 0 ? -(int64_t)lead : (int64_t)lead);
    if (got + len > total)
      return io_fail(std::string("restart record ") + what + " holds more than the " + std::to_string(total) +
                     " bytes the block expects");
    cut(segs, got, len, pcs);
    for (size_t i = 0; i < pcs.size(); ++i) {
      const Piece& p = pcs[i];
      char* dst = segs[p.s].p + p.off;
      if (segs[p.s].dev) {
        // buffer i&1 was last handed to the copy of piece i-2
        if (i >= 2) RCU(cudaEventSynchronize(sg.ev[i & 1]));
        dst = sg.pin[i & 1];
      }
      if (fread(dst, 1, p.len, f) != p.len) return io_fail(std::string("restart file ends inside ") + what);
      if (segs[p.s].dev) {
        RCU(cudaMemcpyAsync(segs[p.s].p + p.off, dst, p.len, cudaMemcpyHostToDevice, sg.st));
        RCU(cudaEventRecord(sg.ev[i & 1], sg.st));
      }
    }
    if (sg.ready) RCU(cudaStreamSynchronize(sg.st));
    got += len;
    if (!get_marker(f, &tail)) return io_fail(std::string("restart file ends inside ") + what);
    const bool tail_ok = (int64_t)(tail < 0 ? -(int64_t)tail : (int64_t)tail) == (int64_t)len &&
                         ((tail < 0) == !first);
    if (!tail_ok) return io_fail(std::string("restart record ") + what + ": corrupt record marker");
    first = false;
    if (lead >= 0) break;
  }
  if (got != total)
    return io_fail(std::string("restart record ") + what + " holds " + std::to_string(got) + " bytes, the block expects " +
                   std::to_string(total));
  return ASAM_OK;
}

int block_segments(const asam_restart_block& b, int ib, std::vector<std::vector<Seg>>& recs) {
  if (b.nx < 1 || b.ny < 1 || b.nz < 1 || b.ncomp < 0 || b.nfrac < 0)
    return arg_fail("restart block " + std::to_string(ib) + ": bad extents");
  if ((b.ncomp > 0 && !b.c) || !b.uf || !b.vf || !b.wf)
    return arg_fail("restart block " + std::to_string(ib) + ": null array");
  const size_t nx = b.nx, ny = b.ny, nz = b.nz, nf = b.nfrac ? b.nfrac : 1;
  const size_t comp = (nx + 2) * (ny + 2) * (nz + 2) * nf * sizeof(double);
  const bool cdev = on_device(b.c);
  for (int ic = 0; ic < b.ncomp; ++ic) recs.push_back({Seg{(char*)b.c + ic * comp, comp, cdev}});
  recs.push_back({Seg{(char*)b.uf, (nx + 1) * ny * nz * sizeof(double), on_device(b.uf)},
                  Seg{(char*)b.vf, nx * (ny + 1) * nz * sizeof(double), on_device(b.vf)},
                  Seg{(char*)b.wf, nx * ny * (nz + 1) * sizeof(double), on_device(b.wf)}});
  return ASAM_OK;
}

int restart_io(const char* path, asam_restart_header* hdr, int nblock, const asam_restart_block* blocks,
               bool write) {
  if (!path || !hdr || nblock < 0 || (nblock > 0 && !blocks)) return arg_fail("restart: null argument");
  std::vector<std::vector<Seg>> recs;
  std::vector<std::string> names;
  for (int ib = 0; ib < nblock; ++ib) {
    size_t before = recs.size();
    int rc = block_segments(blocks[ib], ib, recs);
    if (rc) return rc;
    for (size_t r = before; r + 1 < recs.size(); ++r)
      names.push_back("block " + std::to_string(ib) + " component " + std::to_string(r - before + 1));
    names.push_back("block " + std::to_string(ib) + " face velocity");
  }
  bool any_dev = false;
  for (auto& r : recs)
    for (auto& s : r) any_dev |= s.dev;
  Stage sg;
  if (any_dev) {
    // the state may still be written by kernels on other streams
    RCU(cudaDeviceSynchronize());
    int rc = sg.init();
    if (rc) return rc;
  }
  FILE* f = fopen(path, write ? "wb" : "rb");
  if (!f) return io_fail(std::string("cannot open restart file ") + path + ": " + strerror(errno));
  int32_t gmv = hdr->gmv_step;
  std::vector<std::vector<Seg>> head = {{Seg{(char*)&hdr->time, 8, false}},
                                        {Seg{(char*)&gmv, 4, false}},
                                        {Seg{(char*)&hdr->output_time, 8, false}}};
  const char* hname[3] = {"Time", "GMVStep", "OutputTime"};
  int rc = ASAM_OK;
  for (int k = 0; k < 3 && rc == ASAM_OK; ++k)
    rc = write ? write_record(f, head[k], sg, hname[k]) : read_record(f, head[k], sg, hname[k]);
  for (size_t r = 0; r < recs.size() && rc == ASAM_OK; ++r)
    rc = write ? write_record(f, recs[r], sg, names[r].c_str()) : read_record(f, recs[r], sg, names[r].c_str());
  if (!write && rc == ASAM_OK) hdr->gmv_step = gmv;
  if (fclose(f) != 0 && rc == ASAM_OK) rc = io_fail(std::string("restart file close failed: ") + strerror(errno));
  return rc;
}

}  // namespace

extern "C" {

int asam_restart_write(const char* path, const asam_restart_header* hdr, int nblock,
                       const asam_restart_block* blocks) {
  if (!hdr) return arg_fail("restart: null header");
  asam_restart_header h = *hdr;
  return restart_io(path, &h, nblock, blocks, true);
}

int asam_restart_read(const char* path, asam_restart_header* hdr, int nblock, const asam_restart_block* blocks) {
  return restart_io(path, hdr, nblock, blocks, false);
}

int asam_restart_file_name(const char* grid_file, int rank, char* buf, int cap) {
  if (!grid_file || !buf || cap < 1 || rank < 0) return arg_fail("restart_file_name: bad argument");
  // FileName(1:INDEX(FileName,'.grid')): up to and including the dot of the
  // first ".grid", nothing when there is none; TRIM drops trailing blanks
  std::string g(grid_file);
  size_t at = g.find(".grid");
  std::string stem = at == std::string::npos ? std::string() : g.substr(0, at + 1);
  while (!stem.empty() && stem.back() == ' ') stem.pop_back();
  std::string name = "RESTART/" + stem + std::to_string(rank);
  if ((int)name.size() + 1 > cap) return arg_fail("restart_file_name: buffer too small");
  memcpy(buf, name.c_str(), name.size() + 1);
  return ASAM_OK;
}

int asam_restart_set_max_subrecord(long long bytes) {
  if (bytes < 1 || bytes > kGfortranMaxSubrecord) return arg_fail("restart: subrecord length out of range");
  g_max_subrecord = bytes;
  return ASAM_OK;
}

}  // extern "C"
