// flof_uni.cu -- the reference's .uni grid files (source/fileio.cpp:834-1000):
// gzip streams holding a 4-byte tag ("MNT2" for a 3D Grid<T>, "M4T2" for a
// Grid4d<T>), a 288-byte UniHeader, for 4D an int32 t extent, then the cells
// as float32 (x fastest), one t slice after the other.
//
// zlib is bound at run time (dlopen of libz.so.1), so the build needs no zlib
// headers; on a machine without the library the file entry points fail with
// FLOF_E_ARG and say so.  Files move through two pinned slice buffers: slice
// t+1 is (de)compressed while slice t crosses the host link.
#include <dlfcn.h>
#include <time.h>

#include "flof_internal.h"

using namespace flof;
using namespace fh;

namespace {

// source/fileio.cpp:38-44
struct UniHeader {
  int dimX, dimY, dimZ;
  int gridType, elementType, bytesPerElement;
  char info[256];
  unsigned long long timestamp;
};
static_assert(sizeof(UniHeader) == 288, "UniHeader layout");

// gzip entry points of zlib (zlib.h), bound by name.
struct Zlib {
  void *(*open)(const char *, const char *) = nullptr;
  int (*read)(void *, void *, unsigned) = nullptr;
  int (*write)(void *, const void *, unsigned) = nullptr;
  int (*close)(void *) = nullptr;
  long (*seek)(void *, long, int) = nullptr;
  int (*buffer)(void *, unsigned) = nullptr;
  bool ok = false;
};

const Zlib &zlib() {
  static Zlib z = [] {
    Zlib r;
    void *h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) return r;
    r.open = (void *(*)(const char *, const char *))dlsym(h, "gzopen");
    r.read = (int (*)(void *, void *, unsigned))dlsym(h, "gzread");
    r.write = (int (*)(void *, const void *, unsigned))dlsym(h, "gzwrite");
    r.close = (int (*)(void *))dlsym(h, "gzclose");
    r.seek = (long (*)(void *, long, int))dlsym(h, "gzseek");
    r.buffer = (int (*)(void *, unsigned))dlsym(h, "gzbuffer");
    r.ok = r.open && r.read && r.write && r.close && r.seek;
    return r;
  }();
  return z;
}

const Zlib &need_zlib() {
  const Zlib &z = zlib();
  need(z.ok, "zlib (libz.so.1) is not available: .uni files cannot be read or written");
  return z;
}

struct GzFile {
  void *f = nullptr;
  explicit GzFile(const char *name, const char *mode) {
    const Zlib &z = need_zlib();
    f = z.open(name, mode);
    if (!f) fail(FLOF_E_NOTFOUND, std::string("can't open file ") + name);
    if (z.buffer) z.buffer(f, 1u << 20);
  }
  ~GzFile() {
    if (f) zlib().close(f);
  }
  GzFile(const GzFile &) = delete;
  GzFile &operator=(const GzFile &) = delete;
  // reads exactly n bytes (in pieces below 2^31)
  bool read(void *dst, size_t n) {
    char *p = (char *)dst;
    while (n > 0) {
      const unsigned chunk = (unsigned)(n < (1u << 30) ? n : (1u << 30));
      const int got = zlib().read(f, p, chunk);
      if (got != (int)chunk) return false;
      p += chunk;
      n -= chunk;
    }
    return true;
  }
  void write(const void *src, size_t n) {
    const char *p = (const char *)src;
    while (n > 0) {
      const unsigned chunk = (unsigned)(n < (1u << 30) ? n : (1u << 30));
      if (zlib().write(f, p, chunk) != (int)chunk) fail(FLOF_E_ARG, "gzwrite failed");
      p += chunk;
      n -= chunk;
    }
  }
  void close() {
    if (f && zlib().close(f) != 0) {
      f = nullptr;
      fail(FLOF_E_ARG, "gzclose failed");
    }
    f = nullptr;
  }
};

struct UniFile {
  bool is4d = false;
  UniHeader h;
  int dimT = 1;
};

// Reads the tag and header (and the 4D t extent) of an open file.
UniFile read_header(GzFile &g, const char *name) {
  char id[5] = {0, 0, 0, 0, 0};
  if (!g.read(id, 4)) fail(FLOF_E_ARG, std::string("can't read file ") + name);
  UniFile u;
  if (!strcmp(id, "MNT2")) {
    u.is4d = false;
  } else if (!strcmp(id, "M4T2")) {
    u.is4d = true;
  } else {
    fail(FLOF_E_ARG, std::string(name) + ": unknown header '" + id +
                         "' (supported: MNT2, M4T2 with float32 cells)");
  }
  if (!g.read(&u.h, sizeof(UniHeader))) fail(FLOF_E_ARG, "can't read file, no header present");
  if (u.is4d && !g.read(&u.dimT, sizeof(int))) fail(FLOF_E_ARG, "can't read the t extent");
  return u;
}

// unifyGridType (fileio.cpp:470-479): Real <> Levelset, Vec3 <> MAC.  The
// reference applies it to Grid4d type codes as well, where 8 is Vec4.
int unify(int type) {
  if (type & 1) type |= 16;
  if (type & 16) type |= 1;
  if (type & 4) type |= 8;
  if (type & 8) type |= 4;
  return type;
}

struct Events2 {
  cudaEvent_t e[2] = {nullptr, nullptr};
  Events2() {
    CK(cudaEventCreateWithFlags(&e[0], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&e[1], cudaEventDisableTiming));
  }
  ~Events2() {
    if (e[0]) cudaEventDestroy(e[0]);
    if (e[1]) cudaEventDestroy(e[1]);
  }
};

struct Pinned {
  void *p = nullptr;
  explicit Pinned(size_t n) {
    if (cudaMallocHost(&p, n ? n : 16) != cudaSuccess) {
      cudaGetLastError();
      fail(FLOF_E_OOM, "pinned host allocation failed");
    }
  }
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

// Streams `nslices` slices of `slice_bytes` from the file into device memory
// at dst, two pinned buffers in flight.
void stream_in(flof_ctx *c, GzFile &g, char *dst, size_t slice_bytes, int nslices,
               const char *name) {
  Pinned b0(slice_bytes), b1(slice_bytes);
  Events2 ev;
  void *buf[2] = {b0.p, b1.p};
  bool ok = true;
  for (int t = 0; t < nslices; ++t) {
    const int k = t & 1;
    // buffer k was last handed to the copy of slice t-2
    if (t >= 2) CK(cudaEventSynchronize(ev.e[k]));
    ok = g.read(buf[k], slice_bytes);
    if (!ok) break;
    CK(cudaMemcpyAsync(dst + (size_t)t * slice_bytes, buf[k], slice_bytes,
                       cudaMemcpyHostToDevice, c->stream));
    CK(cudaEventRecord(ev.e[k], c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  if (!ok) fail(FLOF_E_ARG, std::string(name) + ": file ends before its data");
}

void stream_out(flof_ctx *c, GzFile &g, const char *src, size_t slice_bytes, int nslices) {
  Pinned b0(slice_bytes), b1(slice_bytes);
  void *buf[2] = {b0.p, b1.p};
  if (nslices <= 0) return;
  CK(cudaMemcpyAsync(buf[0], src, slice_bytes, cudaMemcpyDeviceToHost, c->stream));
  for (int t = 0; t < nslices; ++t) {
    CK(cudaStreamSynchronize(c->stream));
    if (t + 1 < nslices)
      CK(cudaMemcpyAsync(buf[(t + 1) & 1], src + (size_t)(t + 1) * slice_bytes, slice_bytes,
                         cudaMemcpyDeviceToHost, c->stream));
    g.write(buf[t & 1], slice_bytes);
  }
  CK(cudaStreamSynchronize(c->stream));
}

}  // namespace

namespace fh {

// Loads a 3D (MNT2) or 4D (M4T2) file into g; the file's extents and cell
// size must match g (a 3D file needs a grid with t extent 1).
void uni_load(flof_grid *g, const char *name) {
  GzFile f(name, "rb");
  UniFile u = read_header(f, name);
  const UniHeader &h = u.h;
  need(h.dimX == g->dims[0] && h.dimY == g->dims[1] && h.dimZ == g->dims[2],
       std::string(name) + ": grid dim doesn't match (" + std::to_string(h.dimX) + "," +
           std::to_string(h.dimY) + "," + std::to_string(h.dimZ) + ")");
  need(u.dimT == g->dims[3], std::string(name) + ": t extent " + std::to_string(u.dimT) +
                                 " doesn't match the grid's " + std::to_string(g->dims[3]));
  need(h.bytesPerElement == (int)(g->nc() * sizeof(float)),
       std::string(name) + ": element size " + std::to_string(h.bytesPerElement) +
           " doesn't match the grid's");
  const int want_type = g->elem == FLOF_VEC4 ? 8 : 1;
  need(unify(h.gridType) == unify(want_type),
       std::string(name) + ": grid type " + std::to_string(h.gridType) + " doesn't match");
  const size_t slice = (size_t)g->dims[0] * g->dims[1] * g->dims[2] * g->nc() * sizeof(float);
  set_ctx_device(g->ctx);
  stream_in(g->ctx, f, (char *)g->d, slice, g->dims[3], name);
}

// Writes g as a 4D (is4d) or 3D file like writeGrid4dUni / writeGridUni.
void uni_save(const flof_grid *g, const char *name, bool is4d, int gridType) {
  UniHeader h;
  memset(&h, 0, sizeof(h));
  h.dimX = g->dims[0];
  h.dimY = g->dims[1];
  h.dimZ = g->dims[2];
  h.gridType = gridType;
  h.elementType = g->elem == FLOF_VEC4 ? 2 : 1;
  h.bytesPerElement = (int)(g->nc() * sizeof(float));
  snprintf(h.info, sizeof(h.info), "%s", flof_version());
  h.timestamp = (unsigned long long)time(nullptr) * 1000000ull;
  GzFile f(name, "wb1");
  f.write(is4d ? "M4T2" : "MNT2", 4);
  f.write(&h, sizeof(h));
  if (is4d) {
    const int T = g->dims[3];
    f.write(&T, sizeof(int));
  }
  const size_t slice = (size_t)g->dims[0] * g->dims[1] * g->dims[2] * g->nc() * sizeof(float);
  set_ctx_device(g->ctx);
  stream_out(g->ctx, f, (const char *)g->d, slice, g->dims[3]);
  f.close();
}

// readGrid4dUni with a t slice (fileio.cpp:912-990): slice t of a 4D file
// into a grid with the file's x, y, z extents and t extent 1.
void uni_read_slice(flof_grid *g, const char *name, int t) {
  GzFile f(name, "rb");
  UniFile u = read_header(f, name);
  need(u.is4d, std::string(name) + " is not a 4D (M4T2) file");
  const UniHeader &h = u.h;
  need(h.dimX == g->dims[0] && h.dimY == g->dims[1] && h.dimZ == g->dims[2] &&
           g->dims[3] == 1,
       std::string(name) + ": slice grid dim doesn't match");
  need(h.bytesPerElement == (int)(g->nc() * sizeof(float)),
       std::string(name) + ": element size doesn't match");
  need(t >= 0 && t < u.dimT, std::string(name) + ": grid dim4 slice too large");
  const size_t slice = (size_t)h.dimX * h.dimY * h.dimZ * h.bytesPerElement;
  const long off = (long)(slice * (size_t)t + sizeof(UniHeader) + sizeof(int) + 4);
  need(zlib().seek(f.f, off, SEEK_SET) == off, std::string(name) + ": seek failed");
  set_ctx_device(g->ctx);
  stream_in(g->ctx, f, (char *)g->d, slice, 1, name);
}

UniInfo uni_info(const char *name) {
  GzFile f(name, "rb");
  UniFile u = read_header(f, name);
  UniInfo r;
  r.dims[0] = u.h.dimX;
  r.dims[1] = u.h.dimY;
  r.dims[2] = u.h.dimZ;
  r.dims[3] = u.dimT;
  r.is4d = u.is4d;
  r.gridType = u.h.gridType;
  r.elementType = u.h.elementType;
  r.bytesPerElement = u.h.bytesPerElement;
  return r;
}

}  // namespace fh

// ---- C ABI ------------------------------------------------------------------

FLOF_API int flof_uni_info(const char *fname, int dims[4], int *is4d, int *gridType,
                           int *bytesPerElement) {
  return guarded_host([&] {
    need(fname != nullptr && dims != nullptr, "NULL argument");
    const UniInfo u = uni_info(fname);
    for (int q = 0; q < 4; ++q) dims[q] = u.dims[q];
    if (is4d) *is4d = u.is4d ? 1 : 0;
    if (gridType) *gridType = u.gridType;
    if (bytesPerElement) *bytesPerElement = u.bytesPerElement;
  });
}

FLOF_API int flof_grid_load(flof_grid *g, const char *fname) {
  return guarded([&] {
    need_grid(g, "grid");
    need(fname != nullptr, "file name is NULL");
    uni_load(g, fname);
  });
}

FLOF_API int flof_grid_save(const flof_grid *g, const char *fname, int is4d) {
  return guarded([&] {
    need_grid(g, "grid");
    need(fname != nullptr, "file name is NULL");
    need(is4d || g->dims[3] == 1, "a 3D file needs a grid with t extent 1");
    need(is4d || g->elem == FLOF_REAL, "3D files hold Real grids only");
    uni_save(g, fname, is4d != 0, g->elem == FLOF_VEC4 ? 8 : 1);
  });
}

FLOF_API int flof_uni_read_slice(flof_grid *slice, const char *fname, int t) {
  return guarded([&] {
    need_grid(slice, "slice");
    need(fname != nullptr, "file name is NULL");
    uni_read_slice(slice, fname, t);
  });
}
