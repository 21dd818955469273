// sdf_io.cpp -- the dump of this path's state in SDF, the file format of
// the reference's dumps, written on the host from the run's downloaded
// arrays, and the restart reader that reads it back (end of the file).
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
//  - restart dumps first carry the constants the restart reads back
//    (diagnostics.F90:407-416): "dt", "window_shift_fraction" once the
//    window has started, "x_grid_min" -- real8 constant blocks, the value in
//    the metadata and no data (sdf_output_ru.f90 write_constant_meta);
//  - per species its particles (below);
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
#include <memory>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cylpic.h"

namespace {

constexpr int ID_LEN = 32, STR_LEN = 128;
constexpr int HEADER_LEN = 112, BLOCK_HEADER_LEN = 4 * 4 + 3 * 8 + ID_LEN + STR_LEN;
constexpr int32_t ENDIANNESS = 16911887, SDF_VERSION = 1, SDF_REVISION = 4;
constexpr int32_t BT_PLAIN_MESH = 1, BT_POINT_MESH = 2, BT_PLAIN_VARIABLE = 3, BT_POINT_VARIABLE = 4,
                  BT_CONSTANT = 5;
constexpr int32_t DT_INTEGER8 = 2, DT_REAL8 = 4, GEOM_CARTESIAN = 1;
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

int cyl_sdf_write(const char* path, const cyl_sdf_desc* d, const double* const* arrays,
                  const cyl_sdf_species* species, int32_t nspecies) {
  if (!path || !d || !arrays || d->nx < 1 || d->ny < 1 || d->n_mode < 1 || !(d->dx > 0.0) || !(d->dy > 0.0) ||
      nspecies < 0 || (nspecies > 0 && !species))
    return CYL_ERR_BAD_ARG;
  for (int i = 0; i < nspecies; ++i) {
    const cyl_sdf_species& sp = species[i];
    if (!sp.name || !sp.name[0] || sp.n < 0 ||
        (sp.n > 0 && (!sp.x || !sp.y || !sp.z || !sp.px || !sp.py || !sp.pz || !sp.w || !sp.id)))
      return CYL_ERR_BAD_ARG;
  }
  SdfFile f;
  if (!f.open(path, d->step, d->time, d->restart)) return CYL_ERR_IO;
  if (d->restart) {
    struct Const {
      const char *id, *name;
      double v;
      bool on;
    };
    const Const cs[] = {{"dt", "Time increment", d->dt, d->dt > 0.0},
                        {"window_shift_fraction", "Window Shift Fraction", d->window_shift_fraction,
                         d->window_started != 0},
                        {"x_grid_min", "Minimum grid position", d->x_grid_min, true}};
    for (const Const& c : cs) {
      if (!c.on) continue;
      Block b;
      b.id = c.id;
      b.name = c.name;
      b.blocktype = BT_CONSTANT;
      b.ndims = 1;
      b.meta.f64(c.v);
      if (!f.add(b, nullptr)) return CYL_ERR_IO;
    }
  }
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
  // particles (diagnostics.F90:614-722 write_particle_variable, 3030-3075
  // write_particle_grid): per variable every species' point variable
  // "<var>/<species>" on mesh "grid/<species>", then every species' 3D
  // point mesh (all x, all y, all z); species without particles are left
  // out, as the reference does
  struct PtVar {
    const char *id, *name, *units;
  };
  const PtVar vars[] = {{"weight", "Weight", ""}, {"px", "Px", "kg.m/s"}, {"py", "Py", "kg.m/s"},
                        {"pz", "Pz", "kg.m/s"}, {"id", "ID", "#"}};
  for (int v = 0; v < 5; ++v)
    for (int i = 0; i < nspecies; ++i) {
      const cyl_sdf_species& sp = species[i];
      if (sp.n == 0) continue;
      Block b;
      b.id = std::string(vars[v].id) + "/" + sp.name;
      b.name = std::string("Particles/") + vars[v].name + "/" + sp.name;
      b.blocktype = BT_POINT_VARIABLE;
      b.datatype = v == 4 ? DT_INTEGER8 : DT_REAL8;
      b.ndims = 1;
      b.data_length = sp.n * 8;
      b.meta.f64(1.0);
      b.meta.str(vars[v].units, ID_LEN);
      b.meta.str(std::string("grid/") + sp.name, ID_LEN);
      b.meta.i64(sp.n);
      b.meta.str(sp.name, ID_LEN);
      const void* data = v == 0 ? (const void*)sp.w
                                : v == 1 ? (const void*)sp.px
                                         : v == 2 ? (const void*)sp.py : v == 3 ? (const void*)sp.pz : (const void*)sp.id;
      if (!f.add(b, data)) return CYL_ERR_IO;
    }
  for (int i = 0; i < nspecies; ++i) {
    const cyl_sdf_species& sp = species[i];
    if (sp.n == 0) continue;
    std::vector<double> xyz((size_t)sp.n * 3);
    double mn[3], mx[3];
    const double* src[3] = {sp.x, sp.y, sp.z};
    for (int k = 0; k < 3; ++k) {
      mn[k] = src[k][0];
      mx[k] = src[k][0];
      for (int64_t p = 0; p < sp.n; ++p) {
        const double v = src[k][p];
        xyz[(size_t)k * (size_t)sp.n + (size_t)p] = v;
        if (v < mn[k]) mn[k] = v;
        if (v > mx[k]) mx[k] = v;
      }
    }
    Block b;
    b.id = std::string("grid/") + sp.name;
    b.name = std::string("Grid/Particles/") + sp.name;
    b.blocktype = BT_POINT_MESH;
    b.ndims = 3;
    b.data_length = sp.n * 3 * 8;
    for (int k = 0; k < 3; ++k) b.meta.f64(1.0);
    b.meta.str("X", ID_LEN);
    b.meta.str("Y", ID_LEN);
    b.meta.str("Z", ID_LEN);
    for (int k = 0; k < 3; ++k) b.meta.str("m", ID_LEN);
    b.meta.i32(GEOM_CARTESIAN);
    for (int k = 0; k < 3; ++k) b.meta.f64(mn[k]);
    for (int k = 0; k < 3; ++k) b.meta.f64(mx[k]);
    b.meta.i64(sp.n);
    b.meta.str(sp.name, ID_LEN);
    if (!f.add(b, xyz.data())) return CYL_ERR_IO;
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

// ---------------------------------------------------------------------------
// The restart reader: the block list of an SDF file as restart_data walks it
// (setup.F90:777-1569 with the SDF library's readers, SDF/FORTRAN
// sdf_input_ru.f90 read_block_header, sdf_input_point_ru.f90,
// sdf_input_cartesian_ru.f90): the header, then every block header and its
// metadata along the next-block chain; data are read on demand.
namespace {

struct RBlock {
  std::string id, name, units, mesh_id, species_id;
  int32_t blocktype = 0, datatype = 0, ndims = 0;
  int64_t data_loc = 0, data_length = 0, npoints = 0;
  std::vector<int32_t> dims;
  std::vector<double> extents;
  double value = 0.0;  // a constant block's value
};

// A bounds-checked cursor over a byte buffer.
struct Cursor {
  const char* p;
  size_t n, o = 0;
  bool ok = true;
  void raw(void* dst, size_t k) {
    if (o + k > n) {
      ok = false;
      std::memset(dst, 0, k);
      return;
    }
    std::memcpy(dst, p + o, k);
    o += k;
  }
  int32_t i32() {
    int32_t v;
    raw(&v, 4);
    return v;
  }
  int64_t i64() {
    int64_t v;
    raw(&v, 8);
    return v;
  }
  double f64() {
    double v;
    raw(&v, 8);
    return v;
  }
  // a string field: up to the first NUL, trailing blanks removed
  std::string str(int len) {
    std::string v((size_t)len, '\0');
    raw(&v[0], (size_t)len);
    const size_t z = v.find('\0');
    if (z != std::string::npos) v.resize(z);
    while (!v.empty() && v.back() == ' ') v.pop_back();
    return v;
  }
};

bool starts_with(const std::string& s, const char* p) { return s.compare(0, std::strlen(p), p) == 0; }

const ModeArray* mode_array(int which) {
  for (const ModeArray* g : GROUPS)
    for (int c = 0; c < 3; ++c)
      if (g[c].which == which) return &g[c];
  return nullptr;
}

}  // namespace

struct cyl_sdf_file_s {
  std::FILE* f = nullptr;
  cyl_sdf_info info{};
  std::vector<RBlock> blocks;
  ~cyl_sdf_file_s() {
    if (f) std::fclose(f);
  }
  bool read_at(int64_t loc, void* dst, size_t n) {
    if (loc < 0 || std::fseek(f, (long)loc, SEEK_SET) != 0) return false;
    return std::fread(dst, 1, n, f) == n;
  }
  const RBlock* find(const std::string& id, int32_t blocktype) const {
    for (const RBlock& b : blocks)
      if (b.blocktype == blocktype && b.id == id) return &b;
    return nullptr;
  }
  // the point mesh of a species: species id, else block id "grid/<name>"
  // (find_species_by_id_or_blockid)
  const RBlock* species_mesh(const std::string& name) const {
    for (const RBlock& b : blocks)
      if (b.blocktype == BT_POINT_MESH && b.species_id == name) return &b;
    return find("grid/" + name, BT_POINT_MESH);
  }
};

int cyl_sdf_open(const char* path, cyl_sdf_file* out) {
  if (!path || !out) return CYL_ERR_BAD_ARG;
  *out = nullptr;
  std::unique_ptr<cyl_sdf_file_s> s(new cyl_sdf_file_s);
  s->f = std::fopen(path, "rb");
  if (!s->f) return CYL_ERR_IO;
  char hb[HEADER_LEN];
  if (!s->read_at(0, hb, sizeof(hb)) || std::memcmp(hb, "SDF1", 4) != 0) return CYL_ERR_IO;
  Cursor c{hb, sizeof(hb), 4};
  const int32_t endianness = c.i32(), version = c.i32();
  c.i32();  // revision
  // files of the other byte order are not read
  if (endianness != ENDIANNESS || version != SDF_VERSION) return CYL_ERR_IO;
  const std::string code = c.str(ID_LEN);
  const int64_t first = c.i64();
  c.i64();  // summary location
  c.i32();  // summary size
  const int32_t nblocks = c.i32(), bhl = c.i32(), step = c.i32();
  const double time = c.f64();
  c.i32();
  c.i32();  // job id
  const int32_t slen = c.i32();
  if (!c.ok || slen < 1 || slen > 4096 || bhl != 4 * 4 + 3 * 8 + ID_LEN + slen || nblocks < 0) return CYL_ERR_IO;
  cyl_sdf_info& I = s->info;
  I.step = step;
  I.time = time;
  I.restart = hb[104] ? 1 : 0;
  std::snprintf(I.code_name, sizeof(I.code_name), "%s", code.c_str());
  int64_t at = first;
  std::vector<char> hdr((size_t)bhl), meta;
  for (int k = 0; k < nblocks; ++k) {
    if (!s->read_at(at, hdr.data(), hdr.size())) return CYL_ERR_IO;
    Cursor h{hdr.data(), hdr.size()};
    RBlock r;
    const int64_t next = h.i64();
    r.data_loc = h.i64();
    r.id = h.str(ID_LEN);
    r.data_length = h.i64();
    r.blocktype = h.i32();
    r.datatype = h.i32();
    r.ndims = h.i32();
    r.name = h.str(slen);
    const int32_t info = h.i32();
    if (!h.ok || info < 0 || info > (1 << 24) || r.ndims < 0 || r.ndims > 8 || r.data_length < 0) return CYL_ERR_IO;
    meta.resize((size_t)info);
    if (info > 0 && !s->read_at(at + bhl, meta.data(), meta.size())) return CYL_ERR_IO;
    Cursor m{meta.data(), meta.size()};
    const int nd = r.ndims;
    switch (r.blocktype) {
      case BT_PLAIN_VARIABLE:
        m.f64();
        r.units = m.str(ID_LEN);
        r.mesh_id = m.str(ID_LEN);
        for (int d = 0; d < nd; ++d) r.dims.push_back(m.i32());
        break;
      case BT_PLAIN_MESH:
      case BT_POINT_MESH:
        for (int d = 0; d < nd; ++d) m.f64();
        for (int d = 0; d < 2 * nd; ++d) m.str(ID_LEN);  // labels, units
        m.i32();                                         // geometry
        for (int d = 0; d < 2 * nd; ++d) r.extents.push_back(m.f64());
        if (r.blocktype == BT_PLAIN_MESH) {
          for (int d = 0; d < nd; ++d) r.dims.push_back(m.i32());
        } else {
          r.npoints = m.i64();
          r.species_id = m.str(ID_LEN);
        }
        break;
      case BT_POINT_VARIABLE:
        m.f64();
        r.units = m.str(ID_LEN);
        r.mesh_id = m.str(ID_LEN);
        r.npoints = m.i64();
        r.species_id = m.str(ID_LEN);
        break;
      case BT_CONSTANT:
        if (r.datatype == DT_REAL8) r.value = m.f64();
        else if (r.datatype == DT_INTEGER8) r.value = (double)m.i64();
        else if (r.datatype == 1) r.value = (double)m.i32();  // integer4
        break;
      default:
        break;  // block types this path does not read
    }
    if (!m.ok) return CYL_ERR_IO;
    s->blocks.push_back(r);
    at = next;
  }
  for (const RBlock& b : s->blocks) {
    if (b.blocktype == BT_PLAIN_VARIABLE && b.mesh_id == "mode_grid" && b.dims.size() == 3 && I.nx == 0) {
      I.nx = b.dims[0];
      I.ny = b.dims[1];
      I.n_mode = b.dims[2];
    }
    if (b.blocktype == BT_PLAIN_MESH && b.id == "grid" && b.extents.size() == 4) {
      I.has_grid = 1;
      I.grid_x0 = b.extents[0];
      I.grid_y0 = b.extents[1];
      I.grid_x1 = b.extents[2];
      I.grid_y1 = b.extents[3];
    }
    if (b.blocktype == BT_CONSTANT && b.datatype == DT_REAL8) {
      if (b.id == "dt") {
        I.has_dt = 1;
        I.dt = b.value;
      } else if (b.id == "window_shift_fraction") {
        I.has_window_shift_fraction = 1;
        I.window_shift_fraction = b.value;
      } else if (b.id == "x_grid_min") {
        I.has_x_grid_min = 1;
        I.x_grid_min = b.value;
      }
    }
  }
  *out = s.release();
  return CYL_OK;
}

int cyl_sdf_close(cyl_sdf_file f) {
  delete f;
  return CYL_OK;
}

int cyl_sdf_get_info(cyl_sdf_file f, cyl_sdf_info* out) {
  if (!f || !out) return CYL_ERR_BAD_ARG;
  *out = f->info;
  return CYL_OK;
}

// exm(:, 1-ng:ny+ng-1, :) += file rows 2-ng:ny+ng for the shifted arrays,
// the whole array otherwise (setup.F90:1222-1390); the file holds rows
// 1..ny, so array row j - shift receives file row j.
int cyl_sdf_read_field(cyl_sdf_file f, int32_t which, double* data) {
  if (!f || !data) return CYL_ERR_BAD_ARG;
  const ModeArray* a = mode_array(which);
  const cyl_sdf_info& I = f->info;
  if (!a || I.nx < 1 || I.ny < 1 || I.n_mode < 1) return CYL_ERR_BAD_ARG;
  const int ng = CYL_NG, nxg = I.nx + 2 * ng, nyg = I.ny + 2 * ng;
  const size_t count = (size_t)nxg * nyg * I.n_mode;
  std::memset(data, 0, count * 2 * sizeof(double));
  const int shift = (a->stagger == ST_EXM || a->stagger == ST_ETM) ? 1 : 0;
  std::vector<double> v((size_t)I.nx * I.ny * I.n_mode);
  for (int part = 0; part < 2; ++part) {
    const RBlock* b = f->find(std::string(a->id) + (part ? "_imag" : "_real"), BT_PLAIN_VARIABLE);
    if (!b) continue;
    if (b->datatype != DT_REAL8 || b->dims.size() != 3 || b->dims[0] != I.nx || b->dims[1] != I.ny ||
        b->dims[2] != I.n_mode || b->data_length < (int64_t)(v.size() * 8))
      return CYL_ERR_IO;
    if (!f->read_at(b->data_loc, v.data(), v.size() * 8)) return CYL_ERR_IO;
    size_t k = 0;
    for (int m = 0; m < I.n_mode; ++m)
      for (int j = 1; j <= I.ny; ++j)
        for (int i = 1; i <= I.nx; ++i) {
          const int js = j - shift;
          data[2 * ((size_t)(i + ng - 1) + (size_t)nxg * (size_t)(js + ng - 1) + (size_t)nxg * nyg * m) + part] =
              v[k++];
        }
  }
  return CYL_OK;
}

int cyl_sdf_species_count(cyl_sdf_file f, const char* name, int64_t* n_out) {
  if (!f || !name || !n_out) return CYL_ERR_BAD_ARG;
  const RBlock* m = f->species_mesh(name);
  *n_out = m ? m->npoints : -1;
  return CYL_OK;
}

int cyl_sdf_read_particles(cyl_sdf_file f, const char* name, double* x, double* y, double* z, double* px,
                           double* py, double* pz, double* w, int64_t* id, int64_t* n_inout) {
  if (!f || !name || !n_inout) return CYL_ERR_BAD_ARG;
  const RBlock* mesh = f->species_mesh(name);
  if (!mesh) return CYL_ERR_BAD_ARG;
  const int64_t n = mesh->npoints;
  if (n < 0) return CYL_ERR_IO;
  if (*n_inout < n) return CYL_ERR_CAPACITY;
  if (n > 0 && (!x || !y || !z || !px || !py || !pz || !w || !id)) return CYL_ERR_BAD_ARG;
  const size_t un = (size_t)n;
  // the point mesh: x of every particle, then y, then z (write_point_mesh)
  if (mesh->ndims != 3 || mesh->datatype != DT_REAL8 || mesh->data_length < (int64_t)(un * 24)) return CYL_ERR_IO;
  double* xyz[3] = {x, y, z};
  for (int d = 0; d < 3; ++d)
    if (n > 0 && !f->read_at(mesh->data_loc + (int64_t)(d * un * 8), xyz[d], un * 8)) return CYL_ERR_IO;
  struct Var {
    const char* prefix;
    double* dst;
  };
  const Var vars[] = {{"weight/", w}, {"px/", px}, {"py/", py}, {"pz/", pz}};
  for (const Var& v : vars)
    if (n > 0) std::memset(v.dst, 0, un * 8);
  if (n > 0) std::memset(id, 0, un * 8);
  for (const RBlock& b : f->blocks) {
    if (b.blocktype != BT_POINT_VARIABLE) continue;
    if (b.species_id != name && b.mesh_id != mesh->id) continue;
    const bool is_id = starts_with(b.id, "id/");
    const Var* v = nullptr;
    for (const Var& c : vars)
      if (starts_with(b.id, c.prefix)) v = &c;
    if (!v && !is_id) continue;
    // a variable of another count than its mesh is a malformed dump
    if (b.npoints != n) return CYL_ERR_IO;
    if (n == 0) continue;
    if (v) {
      if (b.datatype != DT_REAL8 || b.data_length < (int64_t)(un * 8) || !f->read_at(b.data_loc, v->dst, un * 8))
        return CYL_ERR_IO;
    } else if (b.datatype == DT_INTEGER8) {
      if (b.data_length < (int64_t)(un * 8) || !f->read_at(b.data_loc, id, un * 8)) return CYL_ERR_IO;
    } else if (b.datatype == 1) {  // integer4 ids (PARTICLE_ID4), widened
      std::vector<int32_t> t(un);
      if (b.data_length < (int64_t)(un * 4) || !f->read_at(b.data_loc, t.data(), un * 4)) return CYL_ERR_IO;
      for (size_t i = 0; i < un; ++i) id[i] = t[i];
    } else {
      return CYL_ERR_IO;
    }
  }
  *n_inout = n;
  return CYL_OK;
}
