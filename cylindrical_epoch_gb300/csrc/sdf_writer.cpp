// sdf_writer.cpp -- the mode fields in SDF, the file format of the
// reference's dumps, written on the host from the run's downloaded arrays.
//
// What is written follows the reference's field dump for the mode arrays:
//  - every mode array as two real8 plain-variable blocks, "<id>_real" and
//    "<id>_imag", of dims (nx, ny, n_mode) in Fortran order, on mesh id
//    "mode_grid", with the reference's names, units and stagger codes
//    (diagnostics.F90:498-560 and write_mode_field, 2033-2110).  The cells
//    written are the interior 1..nx, 1..ny of every mode; for arrays whose
//    stagger is that of Ex or Etheta (Ex, Etheta, Br, Jx, Jtheta and their
//    _old copies) the rows are shifted up by one, so that file row 1 holds
//    the axis row 0 (array_print in write_mode_field);
//  - the 2D plain mesh "grid" of the cell edges xb(1..nx+1), yb(1..ny+1)
//    (diagnostics.F90:870-882, setup.F90:189-200).
// The byte layout is the one of the reference's SDF library (SDF/FORTRAN
// sdf_output_ru.f90 write_header_r8, write_block_header;
// sdf_output_cartesian_ru.f90 write_mesh_meta_r8,
// write_mesh_variable_meta_r8; sdf_output_util.f90 sdf_write_summary):
//  - a 112-byte file header;
//  - per block a 200-byte block header (string length 128), its metadata,
//    then its data;
//  - after the last block a summary repeating every block header and
//    metadata, with the header's summary location, size and block count
//    updated at the end.
// Strings are blank-filled and NUL-terminated when shorter than their field
// minus one, as sdf_safe_write_string_len writes them.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cylpic.h"

namespace {

constexpr int ID_LEN = 32, STR_LEN = 128;
constexpr int HEADER_LEN = 112, BLOCK_HEADER_LEN = 4 * 4 + 3 * 8 + ID_LEN + STR_LEN;
constexpr int32_t ENDIANNESS = 16911887, SDF_VERSION = 1, SDF_REVISION = 4;
constexpr int32_t BT_PLAIN_MESH = 1, BT_PLAIN_VARIABLE = 3, DT_REAL8 = 4, GEOM_CARTESIAN = 1;
constexpr int64_t SUMMARY_OFFSET = 4 + 3 * 4 + ID_LEN + 8;  // where the summary location is in the header

// A byte buffer with the SDF field encodings (native byte order, as the
// reference writes it; the endianness word tells readers which it is).
struct Bytes {
  std::vector<char> b;
  void raw(const void* p, size_t n) { b.insert(b.end(), (const char*)p, (const char*)p + n); }
  void i32(int32_t v) { raw(&v, 4); }
  void i64(int64_t v) { raw(&v, 8); }
  void f64(double v) { raw(&v, 8); }
  void str(const std::string& s, int len) {
    std::string out((size_t)len, ' ');
    const size_t n = s.size() < (size_t)len ? s.size() : (size_t)len;
    std::memcpy(&out[0], s.data(), n);
    if ((int)s.size() + 1 < len)
      for (int i = (int)s.size(); i < len; ++i) out[(size_t)i] = '\0';
    raw(out.data(), out.size());
  }
};

struct Block {
  std::string id, name;
  int32_t blocktype = 0, datatype = DT_REAL8, ndims = 0;
  int64_t data_length = 0;
  Bytes meta;  // the block's metadata after the block header
  int64_t info_length() const { return BLOCK_HEADER_LEN + (int64_t)meta.b.size(); }
};

// Block header + metadata of b, with the given next-block and data locations.
Bytes block_info(const Block& b, int64_t next_block, int64_t data_location) {
  Bytes o;
  o.i64(next_block);
  o.i64(data_location);
  o.str(b.id, ID_LEN);
  o.i64(b.data_length);
  o.i32(b.blocktype);
  o.i32(b.datatype);
  o.i32(b.ndims);
  o.str(b.name, STR_LEN);
  o.i32((int32_t)(b.info_length() - BLOCK_HEADER_LEN));
  o.raw(b.meta.b.data(), b.meta.b.size());
  return o;
}

class SdfFile {
 public:
  bool open(const char* path, int32_t step, double time, int restart) {
    f_ = std::fopen(path, "wb");
    if (!f_) return false;
    Bytes h;
    h.raw("SDF1", 4);
    h.i32(ENDIANNESS);
    h.i32(SDF_VERSION);
    h.i32(SDF_REVISION);
    h.str("Epoch2d", ID_LEN);
    h.i64(HEADER_LEN);  // first block location
    h.i64(HEADER_LEN);  // summary location (updated at close)
    h.i32(0);           // summary size
    h.i32(0);           // blocks
    h.i32(BLOCK_HEADER_LEN);
    h.i32(step);
    h.f64(time);
    h.i32(0);  // job id: start seconds
    h.i32(0);  // job id: start milliseconds
    h.i32(STR_LEN);
    h.i32(1);  // code_io_version
    const char flags[8] = {(char)(restart ? 1 : 0), 0, 0, 0, 0, 0, 0, 0};  // restart, other domains, station
    h.raw(flags, 8);                                                         // file, 5 bytes of padding
    loc_ = HEADER_LEN;
    return put(h) && h.b.size() == (size_t)HEADER_LEN;
  }

  // One block: header and metadata, then its data at the following offset.
  bool add(const Block& b, const void* data) {
    const int64_t start = loc_, data_loc = start + b.info_length(), next = data_loc + b.data_length;
    if (!put(block_info(b, next, data_loc))) return false;
    if (b.data_length > 0 && std::fwrite(data, 1, (size_t)b.data_length, f_) != (size_t)b.data_length) return false;
    blocks_.push_back(b);
    data_locs_.push_back(data_loc);
    loc_ = next;
    return true;
  }

  // The summary after the last block, then the header's summary fields.
  bool close() {
    bool ok = f_ != nullptr;
    const int64_t summary = loc_;
    int64_t at = summary;
    for (size_t i = 0; ok && i < blocks_.size(); ++i) {
      const int64_t next = at + blocks_[i].info_length();
      ok = put(block_info(blocks_[i], next, data_locs_[i]));
      at = next;
    }
    const int32_t size = (int32_t)(at - summary), nblocks = (int32_t)blocks_.size();
    if (ok) ok = std::fseek(f_, (long)SUMMARY_OFFSET, SEEK_SET) == 0;
    if (ok) ok = std::fwrite(&summary, 8, 1, f_) == 1 && std::fwrite(&size, 4, 1, f_) == 1 &&
                 std::fwrite(&nblocks, 4, 1, f_) == 1;
    if (f_ && std::fclose(f_) != 0) ok = false;
    f_ = nullptr;
    return ok;
  }

  ~SdfFile() {
    if (f_) std::fclose(f_);
  }

 private:
  bool put(const Bytes& x) { return std::fwrite(x.b.data(), 1, x.b.size(), f_) == x.b.size(); }
  std::FILE* f_ = nullptr;
  int64_t loc_ = 0;
  std::vector<Block> blocks_;
  std::vector<int64_t> data_locs_;
};

}  // namespace

namespace {

// The mode arrays of the dump in the reference's order, with its ids,
// names, units and stagger codes (constants.F90:291-299: face_x 1,
// face_y 2, edge_z 3, face_z 4).
struct ModeArray {
  int which;
  const char *id, *name, *units;
  int32_t stagger;
  bool restart_only;
};
constexpr int32_t ST_EXM = 2, ST_ERM = 1, ST_ETM = 3, ST_BTM = 4;
const ModeArray E_ARRAYS[] = {
    {CYL_F_EXM, "exm", "Electric Field Modes/Exm", "V/m", ST_EXM, false},
    {CYL_F_ERM, "erm", "Electric Field Modes/Erm", "V/m", ST_ERM, false},
    {CYL_F_ETM, "etm", "Electric Field Modes/Etm", "V/m", ST_ETM, false}};
const ModeArray B_ARRAYS[] = {
    {CYL_F_BXM, "bxm", "Magnetic Field Modes/Bxm", "T", ST_ERM, false},
    {CYL_F_BRM, "brm", "Magnetic Field Modes/Brm", "T", ST_EXM, false},
    {CYL_F_BTM, "btm", "Magnetic Field Modes/Btm", "T", ST_BTM, false}};
const ModeArray BO_ARRAYS[] = {
    {CYL_F_BXM_OLD, "bxm_old", "Magnetic Field Modes/Bxm_old", "T", ST_ERM, true},
    {CYL_F_BRM_OLD, "brm_old", "Magnetic Field Modes/Brm_old", "T", ST_EXM, true},
    {CYL_F_BTM_OLD, "btm_old", "Magnetic Field Modes/Btm_old", "T", ST_BTM, true}};
const ModeArray J_ARRAYS[] = {
    {CYL_F_JXM, "jxm", "Current Modes/Jxm", "A/m^2", ST_EXM, false},
    {CYL_F_JRM, "jrm", "Current Modes/Jrm", "A/m^2", ST_ERM, false},
    {CYL_F_JTM, "jtm", "Current Modes/Jtm", "A/m^2", ST_ETM, false}};
const ModeArray JO_ARRAYS[] = {
    {CYL_F_JXM_OLD, "jxm_old", "Current Modes/Jxm_old", "A/m^2", ST_EXM, true},
    {CYL_F_JRM_OLD, "jrm_old", "Current Modes/Jrm_old", "A/m^2", ST_ERM, true},
    {CYL_F_JTM_OLD, "jtm_old", "Current Modes/Jtm_old", "A/m^2", ST_ETM, true}};
const ModeArray* const GROUPS[] = {E_ARRAYS, B_ARRAYS, BO_ARRAYS, J_ARRAYS, JO_ARRAYS};

// The real or imaginary part (part 0 / 1) of the interior of a mode array
// given in the cyl_download_field layout, in Fortran order; shift 1 puts
// array row j - 1 in file row j (row 1 - ng reads as zero).
std::vector<double> interior(const cyl_sdf_desc& d, const double* a, int part, int shift) {
  const int ng = CYL_NG, nxg = d.nx + 2 * ng, nyg = d.ny + 2 * ng;
  std::vector<double> out((size_t)d.nx * d.ny * d.n_mode);
  size_t k = 0;
  for (int m = 0; m < d.n_mode; ++m)
    for (int j = 1; j <= d.ny; ++j)
      for (int i = 1; i <= d.nx; ++i) {
        const int js = j - shift;
        out[k++] = a[2 * ((size_t)(i + ng - 1) + (size_t)nxg * (size_t)(js + ng - 1) + (size_t)nxg * nyg * m) + part];
      }
  return out;
}

}  // namespace

extern "C" {

int cyl_sdf_write(const char* path, const cyl_sdf_desc* d, const double* const* arrays) {
  if (!path || !d || !arrays || d->nx < 1 || d->ny < 1 || d->n_mode < 1 || !(d->dx > 0.0) || !(d->dy > 0.0))
    return CYL_ERR_BAD_ARG;
  SdfFile f;
  if (!f.open(path, d->step, d->time, d->restart)) return CYL_ERR_IO;
  for (const ModeArray* g : GROUPS) {
    for (int part = 0; part < 2; ++part)
      for (int c = 0; c < 3; ++c) {
        const ModeArray& a = g[c];
        if ((a.restart_only && !d->restart) || !arrays[a.which]) continue;
        const int shift = (a.stagger == ST_EXM || a.stagger == ST_ETM) ? 1 : 0;
        const std::vector<double> v = interior(*d, arrays[a.which], part, shift);
        Block b;
        b.id = std::string(a.id) + (part ? "_imag" : "_real");
        b.name = std::string(a.name) + (part ? "/imag" : "/real");
        b.blocktype = BT_PLAIN_VARIABLE;
        b.ndims = 3;
        b.data_length = (int64_t)v.size() * 8;
        b.meta.f64(1.0);  // mult
        b.meta.str(a.units, ID_LEN);
        b.meta.str("mode_grid", ID_LEN);
        b.meta.i32(d->nx);
        b.meta.i32(d->ny);
        b.meta.i32(d->n_mode);
        b.meta.i32(a.stagger);
        if (!f.add(b, v.data())) return CYL_ERR_IO;
      }
  }
  // the grid of cell edges
  std::vector<double> xy((size_t)(d->nx + 1 + d->ny + 1));
  for (int i = 0; i <= d->nx; ++i) xy[(size_t)i] = d->xb_min + (double)i * d->dx;
  for (int j = 0; j <= d->ny; ++j) xy[(size_t)(d->nx + 1 + j)] = (double)j * d->dy;
  Block g;
  g.id = "grid";
  g.name = "Grid/Grid";
  g.blocktype = BT_PLAIN_MESH;
  g.ndims = 2;
  g.data_length = (int64_t)xy.size() * 8;
  g.meta.f64(1.0);
  g.meta.f64(1.0);
  g.meta.str("X", ID_LEN);
  g.meta.str("Y", ID_LEN);
  g.meta.str("m", ID_LEN);
  g.meta.str("m", ID_LEN);
  g.meta.i32(GEOM_CARTESIAN);
  g.meta.f64(xy[0]);
  g.meta.f64(xy[(size_t)d->nx + 1]);
  g.meta.f64(xy[(size_t)d->nx]);
  g.meta.f64(xy.back());
  g.meta.i32(d->nx + 1);
  g.meta.i32(d->ny + 1);
  if (!f.add(g, xy.data())) return CYL_ERR_IO;
  return f.close() ? CYL_OK : CYL_ERR_IO;
}

}  // extern "C"
