// OpenMOC track files: the reader of src/tracks.c:170-323 (load_OpenMOC_tracks,
// the reference's -d input) as a bounds-checked host reader with a C ABI.
//
// File layout (native byte order, as the reference reads it with fread):
//   int    string_length;  char geometry[string_length]
//   int    n_azimuthal;    double spacing
//   int    num_tracks[n_azimuthal], num_x[n_azimuthal], num_y[n_azimuthal]
//   double azim_weights[n_azimuthal]
//   per azimuthal angle i, per track j < num_tracks[i]:
//     double x0, y0, x1, y1, phi;  int azim_angle_index;  int num_segments
//     per segment: double length;  int material_id;  int region_id
//                  [int mesh_surface_fwd, mesh_surface_bwd   with CMFD data]
//
// Differences from the reference's reader: every count is checked against the
// bytes left in the file (the reference ignores fread's result and sizes a
// stack array by the file's string length), and a short or inconsistent file
// is MOC_ERR_ARG instead of undefined behaviour.  The values are converted as
// the reference converts them: lengths to float, region ids kept as ids.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "simplemoc_gb300.h"

namespace {

struct Reader {
  FILE *f = nullptr;
  int64_t left = 0;                   // bytes not yet read
  bool ok = true;

  explicit Reader(const char *path) {
    f = path ? std::fopen(path, "rb") : nullptr;
    if (!f) {
      ok = false;
      return;
    }
    if (std::fseek(f, 0, SEEK_END) != 0) ok = false;
    const long n = std::ftell(f);
    if (n < 0 || std::fseek(f, 0, SEEK_SET) != 0) ok = false;
    left = n;
  }
  ~Reader() {
    if (f) std::fclose(f);
  }
  bool read(void *dst, int64_t bytes) {
    if (!ok || bytes < 0 || bytes > left) return ok = false;
    if (bytes && std::fread(dst, 1, (size_t)bytes, f) != (size_t)bytes) return ok = false;
    left -= bytes;
    return true;
  }
  bool skip(int64_t bytes) {
    if (!ok || bytes < 0 || bytes > left) return ok = false;
    if (bytes && std::fseek(f, (long)bytes, SEEK_CUR) != 0) return ok = false;
    left -= bytes;
    return true;
  }
  template <typename T>
  bool get(T &v) {
    return read(&v, sizeof(T));
  }
};

constexpr int64_t TRACK_BYTES = 5 * sizeof(double) + 2 * sizeof(int32_t);

struct Header {
  int32_t n_az = 0;
  double spacing = 0.0;
  std::vector<int32_t> num_tracks, num_x, num_y;
  std::vector<double> azim_weights;
  int64_t n_tracks = 0;
};

int read_header(Reader &r, Header &h) {
  int32_t len = 0;
  if (!r.get(len) || len < 0 || !r.skip(len)) return MOC_ERR_ARG;     // geometry string
  if (!r.get(h.n_az) || h.n_az < 1 || (int64_t)h.n_az * 20 > r.left) return MOC_ERR_ARG;
  if (!r.get(h.spacing)) return MOC_ERR_ARG;
  h.num_tracks.resize((size_t)h.n_az);
  h.num_x.resize((size_t)h.n_az);
  h.num_y.resize((size_t)h.n_az);
  h.azim_weights.resize((size_t)h.n_az);
  if (!r.read(h.num_tracks.data(), 4 * (int64_t)h.n_az) ||
      !r.read(h.num_x.data(), 4 * (int64_t)h.n_az) ||
      !r.read(h.num_y.data(), 4 * (int64_t)h.n_az) ||
      !r.read(h.azim_weights.data(), 8 * (int64_t)h.n_az))
    return MOC_ERR_ARG;
  for (int32_t t : h.num_tracks) {
    if (t < 0) return MOC_ERR_ARG;
    h.n_tracks += t;
  }
  if (h.n_tracks * TRACK_BYTES > r.left) return MOC_ERR_ARG;
  return MOC_OK;
}

}  // namespace

extern "C" {

int moc_openmoc_probe(const char *path, int cmfd, int32_t *n_azimuthal, double *spacing,
                      int64_t *n_tracks_2d, int64_t *n_segments) {
  Reader r(path);
  if (!r.ok) return MOC_ERR_ARG;
  Header h;
  int rc = read_header(r, h);
  if (rc != MOC_OK) return rc;
  const int64_t seg_bytes = 16 + (cmfd ? 8 : 0);
  int64_t total = 0;
  for (int64_t t = 0; t < h.n_tracks; ++t) {
    int32_t ns = 0;
    if (!r.skip(TRACK_BYTES - 4) || !r.get(ns) || ns < 0) return MOC_ERR_ARG;
    if (!r.skip(ns * seg_bytes)) return MOC_ERR_ARG;
    total += ns;
  }
  if (n_azimuthal) *n_azimuthal = h.n_az;
  if (spacing) *spacing = h.spacing;
  if (n_tracks_2d) *n_tracks_2d = h.n_tracks;
  if (n_segments) *n_segments = total;
  return MOC_OK;
}

int moc_openmoc_read(const char *path, int cmfd, int64_t n_tracks_2d, int64_t n_segments,
                     int32_t *num_tracks, int32_t *num_x, int32_t *num_y,
                     double *azim_weights, double *track_geometry, int32_t *azim_index,
                     int64_t *seg_off, float *seg_len, int32_t *material_id,
                     int32_t *region_id) {
  Reader r(path);
  if (!r.ok) return MOC_ERR_ARG;
  Header h;
  int rc = read_header(r, h);
  if (rc != MOC_OK) return rc;
  if (h.n_tracks != n_tracks_2d) return MOC_ERR_ARG;
  for (int32_t i = 0; i < h.n_az; ++i) {
    if (num_tracks) num_tracks[i] = h.num_tracks[(size_t)i];
    if (num_x) num_x[i] = h.num_x[(size_t)i];
    if (num_y) num_y[i] = h.num_y[(size_t)i];
    if (azim_weights) azim_weights[i] = h.azim_weights[(size_t)i];
  }
  int64_t seg = 0;
  if (seg_off) seg_off[0] = 0;
  for (int64_t t = 0; t < h.n_tracks; ++t) {
    double geo[5];
    int32_t ai = 0, ns = 0;
    if (!r.read(geo, sizeof geo) || !r.get(ai) || !r.get(ns) || ns < 0) return MOC_ERR_ARG;
    if (seg + ns > n_segments) return MOC_ERR_ARG;
    if (track_geometry) std::memcpy(track_geometry + 5 * t, geo, sizeof geo);
    if (azim_index) azim_index[t] = ai;
    for (int32_t s = 0; s < ns; ++s, ++seg) {
      double length = 0.0;
      int32_t mat = 0, reg = 0;
      if (!r.get(length) || !r.get(mat) || !r.get(reg)) return MOC_ERR_ARG;
      if (cmfd && !r.skip(8)) return MOC_ERR_ARG;
      if (seg_len) seg_len[seg] = (float)length;            // src/tracks.c:297
      if (material_id) material_id[seg] = mat;
      if (region_id) region_id[seg] = reg;                  // src/tracks.c:300
    }
    if (seg_off) seg_off[t + 1] = seg;
  }
  if (seg != n_segments) return MOC_ERR_ARG;
  return MOC_OK;
}

}  // extern "C"
