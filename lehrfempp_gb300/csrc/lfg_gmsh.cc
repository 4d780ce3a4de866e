// Gmsh reader: GmshReader(factory, filename) of lf::io (io/gmsh_reader.cc,
// io/gmsh_file_v2.cc, io/gmsh_file_v4*.cc) for the 2D first-order meshes of
// this path.  Host code: the file is read and parsed on the host, then the
// MeshFactory input it describes (main nodes in file order, cells, segment
// elements as pre-registered edges) is handed to lfg_mesh_create, which
// numbers edges and builds the topology on the device.
//
// Formats: MSH 2.2 and 4.1, ASCII and binary (either byte order).  Element
// types: points (15), 2-node segments (1), 3-node triangles (2), 4-node
// quadrilaterals (3).  Second-order types (8, 9, 10, 16) describe curved
// cells (TriaO2 / QuadO2 / SegmentO2 geometry), which this TriaO1 / QuadO1
// path does not carry: they are rejected with LFG_UNSUPPORTED, as is every
// other type.  Physical entity numbers follow the reference: per entity the
// numbers of all file elements that map to it (consecutive duplicates of an
// element merge into one entity), from the element (2.2) or from its model
// entity's $Entities record (4.1; $PartitionedEntities for a partitioned
// file).  $Periodic and $GhostElements are read past and ignored, as in the
// reference.
#include <algorithm>
#include <charconv>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/lfg.h"

namespace {

thread_local std::string g_gmsh_error;

struct GmshError {
  lfg_status code;
  std::string msg;
};

[[noreturn]] void Throw(lfg_status code, const std::string& msg) { throw GmshError{code, msg}; }

// Node count of the element types the reader knows; 0 = unknown type.
int NumNodesOf(int type) {
  switch (type) {
    case 1: return 2;    // EDGE2
    case 2: return 3;    // TRIA3
    case 3: return 4;    // QUAD4
    case 8: return 3;    // EDGE3
    case 9: return 6;    // TRIA6
    case 10: return 9;   // QUAD9
    case 15: return 1;   // POINT
    case 16: return 8;   // QUAD8
  }
  return 0;
}
int DimOfType(int type) {
  switch (type) {
    case 15: return 0;
    case 1: case 8: return 1;
    default: return 2;
  }
}
int MainNodesOf(int type) {
  switch (type) {
    case 15: return 1;
    case 1: case 8: return 2;
    case 2: case 9: return 3;
    default: return 4;
  }
}

// --------------------------------------------------------------- the file
struct PhysName {
  int dim;
  int nr;
  std::string name;
};

struct GmshFile {
  int version = 0;  // 2 or 4
  bool binary = false;
  std::vector<PhysName> names;
  // 4.1 model entities: physical tags per (dim, tag); a partitioned file
  // takes them from its partitioned entities instead
  std::map<std::pair<int, int>, std::vector<int>> entity_phys;
  std::map<std::pair<int, int>, std::vector<int>> part_entity_phys;
  int64_t num_partitions = 0;
  // nodes in file order
  std::vector<int64_t> node_tag;
  std::vector<double> node_xyz;  // 3 per node
  // elements in file order (4.1: block after block)
  std::vector<int32_t> el_type;
  std::vector<int32_t> el_phys;     // 2.2: physical number (tag 1)
  std::vector<int32_t> el_block;    // 4.1: block index
  std::vector<int64_t> el_off;      // node list offsets (size n + 1)
  std::vector<int64_t> el_nodes;
  // 4.1 blocks: (entity dim, entity tag)
  std::vector<std::pair<int, int>> blocks;
};

// Cursor over the file bytes.
class Reader {
 public:
  Reader(const char* b, const char* e, const std::string& name) : p_(b), e_(e), name_(name) {}
  bool AtEnd() const { return p_ >= e_; }
  const char* pos() const { return p_; }
  void SkipSpace() {
    while (p_ < e_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\r' || *p_ == '\n')) ++p_;
  }
  void SkipLine() {
    while (p_ < e_ && *p_ != '\n') ++p_;
    if (p_ < e_) ++p_;
  }
  std::string Word() {
    SkipSpace();
    const char* s = p_;
    while (p_ < e_ && !(*p_ == ' ' || *p_ == '\t' || *p_ == '\r' || *p_ == '\n')) ++p_;
    return std::string(s, p_);
  }
  int64_t Int() {
    SkipSpace();
    int64_t v = 0;
    auto r = std::from_chars(p_, e_, v);
    if (r.ec != std::errc()) Fail("an integer");
    p_ = r.ptr;
    return v;
  }
  double Double() {
    SkipSpace();
    double v = 0.0;
    auto r = std::from_chars(p_, e_, v);
    if (r.ec != std::errc()) Fail("a number");
    p_ = r.ptr;
    return v;
  }
  std::string Quoted() {
    SkipSpace();
    if (p_ >= e_ || *p_ != '"') Fail("a quoted name");
    const char* s = ++p_;
    while (p_ < e_ && *p_ != '"') ++p_;
    if (p_ >= e_) Fail("a closing quote");
    std::string r(s, p_);
    ++p_;
    return r;
  }
  void Expect(const char* word) {
    const std::string w = Word();
    if (w != word) Fail(std::string("'") + word + "'");
  }
  // binary: raw little/big-endian values
  template <class T>
  T Bin(bool swap) {
    if (e_ - p_ < static_cast<ptrdiff_t>(sizeof(T))) Fail("more binary data");
    unsigned char b[sizeof(T)];
    std::memcpy(b, p_, sizeof(T));
    if (swap) std::reverse(b, b + sizeof(T));
    T v;
    std::memcpy(&v, b, sizeof(T));
    p_ += sizeof(T);
    return v;
  }
  // size_t fields of the given width
  int64_t Size(int width, bool swap) {
    if (width == 8) return static_cast<int64_t>(Bin<uint64_t>(swap));
    if (width == 4) return static_cast<int64_t>(Bin<uint32_t>(swap));
    Fail("a supported data size");
  }
  // after binary data: the newline before $End...
  void EndBinary(const char* end_word) {
    SkipSpace();
    Expect(end_word);
  }
  void Skip(int64_t bytes) {
    if (bytes < 0 || e_ - p_ < bytes) Fail("more binary data");
    p_ += bytes;
  }
  [[noreturn]] void Fail(const std::string& what) const {
    std::string near(p_, std::min<ptrdiff_t>(e_ - p_, 40));
    for (char& c : near)
      if (static_cast<unsigned char>(c) < 32 || static_cast<unsigned char>(c) > 126) c = '.';
    Throw(LFG_IO_ERROR, "Could not parse file " + name_ + ": expected " + what + " near \"" + near + "\"");
  }

 private:
  const char* p_;
  const char* e_;
  std::string name_;
};

void CheckCount(Reader& r, int64_t n, int64_t limit, const char* what) {
  if (n < 0 || n > limit) r.Fail(std::string("a valid ") + what);
}

// --------------------------------------------------------- MSH 2.2 sections
void ReadNodesV2(Reader& r, GmshFile& f, bool swap) {
  const int64_t n = r.Int();
  CheckCount(r, n, int64_t(1) << 40, "node count");
  f.node_tag.resize(n);
  f.node_xyz.resize(3 * n);
  if (!f.binary) {
    for (int64_t i = 0; i < n; ++i) {
      f.node_tag[i] = r.Int();
      for (int d = 0; d < 3; ++d) f.node_xyz[3 * i + d] = r.Double();
    }
  } else {
    r.SkipLine();
    for (int64_t i = 0; i < n; ++i) {
      f.node_tag[i] = r.Bin<int32_t>(swap);
      for (int d = 0; d < 3; ++d) f.node_xyz[3 * i + d] = r.Bin<double>(swap);
    }
  }
  r.EndBinary("$EndNodes");
}

void AddElement(GmshFile& f, int type, int phys, int block) {
  f.el_type.push_back(type);
  f.el_phys.push_back(phys);
  f.el_block.push_back(block);
  f.el_off.push_back(static_cast<int64_t>(f.el_nodes.size()));
}

int CheckType(Reader& r, int64_t type) {
  const int nn = type > 0 && type < 1000 ? NumNodesOf(static_cast<int>(type)) : 0;
  if (nn == 0)
    Throw(LFG_UNSUPPORTED, "Gmsh element type " + std::to_string(type) + " not supported by the GmshReader of "
                           "this 2D first-order path");
  (void)r;
  return nn;
}

void ReadElementsV2(Reader& r, GmshFile& f, bool swap) {
  const int64_t n = r.Int();
  CheckCount(r, n, int64_t(1) << 40, "element count");
  f.el_off.reserve(n + 1);
  if (!f.binary) {
    for (int64_t i = 0; i < n; ++i) {
      r.Int();  // element number
      const int64_t type = r.Int();
      const int nn = CheckType(r, type);
      const int64_t ntags = r.Int();
      if (ntags < 2) r.Fail("at least two tags (physical, elementary)");
      CheckCount(r, ntags, 1 << 20, "tag count");
      const int phys = static_cast<int>(r.Int());
      for (int64_t t = 1; t < ntags; ++t) r.Int();  // elementary, partitions
      AddElement(f, static_cast<int>(type), phys, 0);
      for (int k = 0; k < nn; ++k) f.el_nodes.push_back(r.Int());
    }
  } else {
    r.SkipLine();
    int64_t done = 0;
    while (done < n) {
      const int32_t type = r.Bin<int32_t>(swap);
      const int32_t count = r.Bin<int32_t>(swap);
      const int32_t ntags = r.Bin<int32_t>(swap);
      const int nn = CheckType(r, type);
      if (count <= 0 || count > n - done || ntags < 2) r.Fail("a valid element group header");
      for (int32_t e = 0; e < count; ++e) {
        r.Bin<int32_t>(swap);  // element number
        const int phys = r.Bin<int32_t>(swap);
        for (int32_t t = 1; t < ntags; ++t) r.Bin<int32_t>(swap);
        AddElement(f, type, phys, 0);
        for (int k = 0; k < nn; ++k) f.el_nodes.push_back(r.Bin<int32_t>(swap));
      }
      done += count;
    }
  }
  f.el_off.push_back(static_cast<int64_t>(f.el_nodes.size()));
  r.EndBinary("$EndElements");
}

// --------------------------------------------------------- MSH 4.1 sections
void ReadEntitiesV4(Reader& r, GmshFile& f, bool swap, int dsize) {
  int64_t num[4];
  if (!f.binary) {
    for (auto& x : num) x = r.Int();
  } else {
    r.SkipLine();
    for (auto& x : num) x = r.Size(dsize, swap);
  }
  for (int dim = 0; dim < 4; ++dim) {
    CheckCount(r, num[dim], int64_t(1) << 32, "entity count");
    for (int64_t i = 0; i < num[dim]; ++i) {
      int tag;
      std::vector<int> phys;
      if (!f.binary) {
        tag = static_cast<int>(r.Int());
        for (int k = 0; k < (dim == 0 ? 3 : 6); ++k) r.Double();
        const int64_t np = r.Int();
        CheckCount(r, np, 1 << 20, "physical tag count");
        for (int64_t k = 0; k < np; ++k) phys.push_back(static_cast<int>(r.Int()));
        if (dim > 0) {
          const int64_t nb = r.Int();
          CheckCount(r, nb, int64_t(1) << 32, "bounding entity count");
          for (int64_t k = 0; k < nb; ++k) r.Int();
        }
      } else {
        tag = r.Bin<int32_t>(swap);
        for (int k = 0; k < (dim == 0 ? 3 : 6); ++k) r.Bin<double>(swap);
        const int64_t np = r.Size(dsize, swap);
        CheckCount(r, np, 1 << 20, "physical tag count");
        for (int64_t k = 0; k < np; ++k) phys.push_back(r.Bin<int32_t>(swap));
        if (dim > 0) {
          const int64_t nb = r.Size(dsize, swap);
          CheckCount(r, nb, int64_t(1) << 32, "bounding entity count");
          r.Skip(nb * 4);
        }
      }
      f.entity_phys[{dim, tag}] = std::move(phys);
    }
  }
  r.EndBinary("$EndEntities");
}

// $PartitionedEntities (4.1): numPartitions, ghost entities, then per
// dimension entities carrying parent and partition lists before the fields of
// a model entity.
void ReadPartitionedEntitiesV4(Reader& r, GmshFile& f, bool swap, int dsize) {
  auto count = [&]() { return f.binary ? r.Size(dsize, swap) : r.Int(); };
  auto i32 = [&]() { return f.binary ? static_cast<int64_t>(r.Bin<int32_t>(swap)) : r.Int(); };
  auto dbl = [&]() { return f.binary ? r.Bin<double>(swap) : r.Double(); };
  if (f.binary) r.SkipLine();
  f.num_partitions = count();
  const int64_t nghost = count();
  CheckCount(r, nghost, int64_t(1) << 32, "ghost entity count");
  for (int64_t i = 0; i < nghost; ++i) {
    i32();
    i32();
  }
  int64_t num[4];
  for (auto& x : num) x = count();
  for (int dim = 0; dim < 4; ++dim) {
    CheckCount(r, num[dim], int64_t(1) << 32, "entity count");
    for (int64_t i = 0; i < num[dim]; ++i) {
      const int tag = static_cast<int>(i32());
      i32();  // parent dim
      i32();  // parent tag
      const int64_t np = count();
      CheckCount(r, np, int64_t(1) << 32, "partition count");
      for (int64_t k = 0; k < np; ++k) i32();
      for (int k = 0; k < (dim == 0 ? 3 : 6); ++k) dbl();
      const int64_t nph = count();
      CheckCount(r, nph, 1 << 20, "physical tag count");
      std::vector<int> phys;
      for (int64_t k = 0; k < nph; ++k) phys.push_back(static_cast<int>(i32()));
      if (dim > 0) {
        const int64_t nb = count();
        CheckCount(r, nb, int64_t(1) << 32, "bounding entity count");
        for (int64_t k = 0; k < nb; ++k) i32();
      }
      f.part_entity_phys[{dim, tag}] = std::move(phys);
    }
  }
  r.EndBinary("$EndPartitionedEntities");
}

void ReadNodesV4(Reader& r, GmshFile& f, bool swap, int dsize) {
  int64_t nblocks, nnodes;
  if (!f.binary) {
    nblocks = r.Int();
    nnodes = r.Int();
    r.Int();
    r.Int();
  } else {
    r.SkipLine();
    nblocks = r.Size(dsize, swap);
    nnodes = r.Size(dsize, swap);
    r.Size(dsize, swap);
    r.Size(dsize, swap);
  }
  CheckCount(r, nnodes, int64_t(1) << 40, "node count");
  CheckCount(r, nblocks, int64_t(1) << 40, "node block count");
  f.node_tag.reserve(nnodes);
  f.node_xyz.reserve(3 * nnodes);
  for (int64_t b = 0; b < nblocks; ++b) {
    int64_t edim, param, n;
    if (!f.binary) {
      edim = r.Int();
      r.Int();
      param = r.Int();
      n = r.Int();
    } else {
      edim = r.Bin<int32_t>(swap);
      r.Bin<int32_t>(swap);
      param = r.Bin<int32_t>(swap);
      n = r.Size(dsize, swap);
    }
    CheckCount(r, n, nnodes - static_cast<int64_t>(f.node_tag.size()), "node block size");
    const int extra = param ? static_cast<int>(std::max<int64_t>(0, std::min<int64_t>(edim, 3))) : 0;
    for (int64_t i = 0; i < n; ++i) f.node_tag.push_back(f.binary ? r.Size(dsize, swap) : r.Int());
    for (int64_t i = 0; i < n; ++i) {
      for (int d = 0; d < 3; ++d) f.node_xyz.push_back(f.binary ? r.Bin<double>(swap) : r.Double());
      for (int d = 0; d < extra; ++d) f.binary ? r.Bin<double>(swap) : r.Double();
    }
  }
  if (static_cast<int64_t>(f.node_tag.size()) != nnodes) r.Fail("the announced number of nodes");
  r.EndBinary("$EndNodes");
}

void ReadElementsV4(Reader& r, GmshFile& f, bool swap, int dsize) {
  int64_t nblocks, nel;
  if (!f.binary) {
    nblocks = r.Int();
    nel = r.Int();
    r.Int();
    r.Int();
  } else {
    r.SkipLine();
    nblocks = r.Size(dsize, swap);
    nel = r.Size(dsize, swap);
    r.Size(dsize, swap);
    r.Size(dsize, swap);
  }
  CheckCount(r, nel, int64_t(1) << 40, "element count");
  CheckCount(r, nblocks, int64_t(1) << 40, "element block count");
  f.el_off.reserve(nel + 1);
  for (int64_t b = 0; b < nblocks; ++b) {
    int64_t edim, etag, type, n;
    if (!f.binary) {
      edim = r.Int();
      etag = r.Int();
      type = r.Int();
      n = r.Int();
    } else {
      edim = r.Bin<int32_t>(swap);
      etag = r.Bin<int32_t>(swap);
      type = r.Bin<int32_t>(swap);
      n = r.Size(dsize, swap);
    }
    const int nn = CheckType(r, type);
    if (edim != DimOfType(static_cast<int>(type))) r.Fail("an element block whose dimension matches its type");
    CheckCount(r, n, nel - static_cast<int64_t>(f.el_type.size()), "element block size");
    f.blocks.emplace_back(static_cast<int>(edim), static_cast<int>(etag));
    const int bi = static_cast<int>(f.blocks.size() - 1);
    for (int64_t e = 0; e < n; ++e) {
      f.binary ? r.Size(dsize, swap) : r.Int();  // element tag
      AddElement(f, static_cast<int>(type), 0, bi);
      for (int k = 0; k < nn; ++k) f.el_nodes.push_back(f.binary ? r.Size(dsize, swap) : r.Int());
    }
  }
  if (static_cast<int64_t>(f.el_type.size()) != nel) r.Fail("the announced number of elements");
  f.el_off.push_back(static_cast<int64_t>(f.el_nodes.size()));
  r.EndBinary("$EndElements");
}

void ReadPhysicalNames(Reader& r, GmshFile& f) {
  const int64_t n = r.Int();
  CheckCount(r, n, 1 << 24, "physical name count");
  for (int64_t i = 0; i < n; ++i) {
    PhysName p;
    p.dim = static_cast<int>(r.Int());
    p.nr = static_cast<int>(r.Int());
    p.name = r.Quoted();
    f.names.push_back(std::move(p));
  }
  r.Expect("$EndPhysicalNames");
}

// Skip an unknown or ignored section: everything up to its $End line.
void SkipSection(Reader& r, const std::string& name, const char* end) {
  const std::string marker = "$End" + name.substr(1);
  const char* p = r.pos();
  const char* hit = nullptr;
  for (const char* q = p; q + marker.size() <= end; ++q) {
    if (*q == '$' && std::memcmp(q, marker.data(), marker.size()) == 0) {
      hit = q;
      break;
    }
  }
  if (!hit) r.Fail(marker);
  r.Skip(hit - p + static_cast<int64_t>(marker.size()));
}

GmshFile Parse(const char* data, size_t size, const std::string& name) {
  GmshFile f;
  const char* end = data + size;
  Reader r(data, end, name);
  r.Expect("$MeshFormat");
  const std::string ver = r.Word();
  const int64_t ftype = r.Int();
  const int64_t dsize = r.Int();
  bool swap = false;
  if (ver == "2.2") f.version = 2;
  else if (ver == "4.1") f.version = 4;
  else Throw(LFG_UNSUPPORTED, "GmshFiles with Version " + ver + " are not yet supported.");
  if (ftype != 0 && ftype != 1) r.Fail("file-type 0 or 1");
  f.binary = ftype == 1;
  if (dsize != 8) r.Fail("data-size 8");
  if (f.binary) {
    r.SkipLine();
    const int32_t one = r.Bin<int32_t>(false);
    if (one == 1) swap = false;
    else if (one == 0x01000000) swap = true;
    else r.Fail("the binary one");
  }
  r.Expect("$EndMeshFormat");
  bool have_nodes = false, have_elements = false;
  while (true) {
    r.SkipSpace();
    if (r.AtEnd()) break;
    const std::string sec = r.Word();
    if (sec == "$PhysicalNames") {
      ReadPhysicalNames(r, f);
    } else if (sec == "$Entities" && f.version == 4) {
      ReadEntitiesV4(r, f, swap, static_cast<int>(dsize));
    } else if (sec == "$PartitionedEntities" && f.version == 4) {
      ReadPartitionedEntitiesV4(r, f, swap, static_cast<int>(dsize));
    } else if (sec == "$Nodes") {
      if (f.version == 2) ReadNodesV2(r, f, swap);
      else ReadNodesV4(r, f, swap, static_cast<int>(dsize));
      have_nodes = true;
    } else if (sec == "$Elements") {
      if (f.version == 2) ReadElementsV2(r, f, swap);
      else ReadElementsV4(r, f, swap, static_cast<int>(dsize));
      have_elements = true;
    } else if (!sec.empty() && sec[0] == '$') {
      SkipSection(r, sec, end);  // $Periodic, $GhostElements, $NodeData, comments
    } else {
      r.Fail("a section");
    }
  }
  if (!have_nodes || !have_elements) Throw(LFG_IO_ERROR, "Could not parse file " + name + ": no $Nodes/$Elements");
  return f;
}

}  // namespace

// ------------------------------------------------------------ the reader
struct lfg_gmsh {
  GmshFile file;
  // MeshFactory input
  std::vector<double> xy;
  std::vector<int32_t> cells;   // 4 per cell
  std::vector<int32_t> edges;   // 2 per pre-registered edge
  // physical numbers per entity of each codim (0 cells, 1 pre-registered edges, 2 nodes)
  std::vector<int64_t> phys_off[3];
  std::vector<int32_t> phys_nr[3];
  // name tables: (nr, codim) pairs per name and (name, codim) per nr, file order
  std::multimap<std::string, std::pair<int, int>> name2nr;
  std::multimap<int, std::pair<std::string, int>> nr2name;
};

namespace {

// GmshReader::InitGmshFile (gmsh_reader.cc:116-325 for 2.2, 327-620 for 4.1)
// with dim_mesh = dim_world = 2.
void Build(lfg_gmsh& g) {
  const GmshFile& f = g.file;
  const int64_t ne = static_cast<int64_t>(f.el_type.size());
  const int64_t nn = static_cast<int64_t>(f.node_tag.size());
  int64_t max_tag = 0;
  for (int64_t t : f.node_tag) max_tag = std::max(max_tag, t);
  for (int64_t t : f.el_nodes) max_tag = std::max(max_tag, t);
  int64_t min_tag = 0;  // 2.2 indexes by node number
  if (f.version == 4 && nn > 0) {
    min_tag = f.node_tag[0];
    for (int64_t t : f.node_tag) min_tag = std::min(min_tag, t);
  }
  for (int64_t t : f.el_nodes)
    if (t < min_tag) Throw(LFG_IO_ERROR, "element references node " + std::to_string(t) + " that the file lacks");
  const int64_t span = max_tag - min_tag + 1;
  if (span > (int64_t(1) << 34)) Throw(LFG_IO_ERROR, "node tags span too large a range");
  // main nodes: the corners of the elements (2.2: every non-point element;
  // 4.1: the elements of dimension 2 only)
  std::vector<uint8_t> main(span, 0);
  int64_t ncells = 0;
  for (int64_t e = 0; e < ne; ++e) {
    const int t = f.el_type[e];
    const int d = DimOfType(t);
    if (d == 2) ++ncells;
    const bool mark = f.version == 2 ? t != 15 : d == 2;
    if (!mark) continue;
    for (int k = 0; k < MainNodesOf(t); ++k) main[f.el_nodes[f.el_off[e] + k] - min_tag] = 1;
  }
  if (ncells == 0) Throw(LFG_IO_ERROR, "MshFile contains no elements with dimension 2");
  std::vector<int64_t> tag2mi(span, -1);
  g.xy.clear();
  for (int64_t i = 0; i < nn; ++i) {
    const int64_t t = f.node_tag[i] - min_tag;
    if (t < 0 || t >= span) continue;
    if (!main[t]) continue;
    if (f.node_xyz[3 * i + 2] != 0.0)
      Throw(LFG_IO_ERROR, "In a 2D GmshMesh, the z-coordinate of every node must be zero");
    tag2mi[t] = static_cast<int64_t>(g.xy.size() / 2);
    g.xy.push_back(f.node_xyz[3 * i]);
    g.xy.push_back(f.node_xyz[3 * i + 1]);
  }
  // element list -> entities, merging consecutive duplicates
  // (2.2: same type and node list; 4.1: same node list within a block)
  std::vector<std::vector<int64_t>> src[3];  // per codim, per entity: contributing elements
  std::vector<std::vector<int64_t>>& node_src = src[2];
  int64_t begin = 0;
  for (int64_t e = 0; e < ne; ++e) {
    const int t = f.el_type[e];
    const int codim = 2 - DimOfType(t);
    const int64_t nb = f.el_off[begin + 0], ee = f.el_off[e];
    const int64_t len_b = f.el_off[begin + 1] - nb, len_e = f.el_off[e + 1] - ee;
    const bool same_group = f.version == 2 ? f.el_type[begin] == t : f.el_block[begin] == f.el_block[e];
    if (e != begin && same_group && len_b == len_e &&
        std::equal(f.el_nodes.begin() + nb, f.el_nodes.begin() + nb + len_b, f.el_nodes.begin() + ee)) {
      if (codim == 2) {
        // the reference appends to the last entity record of codim 2
        if (!node_src.empty()) node_src.back().push_back(e);
      } else {
        src[codim].back().push_back(e);
      }
      continue;
    }
    begin = e;
    if (t == 15) {
      const int64_t mi = tag2mi[f.el_nodes[ee] - min_tag];
      if (mi >= 0) {
        if (static_cast<int64_t>(node_src.size()) <= mi) node_src.resize(mi + 1);
        node_src[mi].push_back(e);
      }
      continue;
    }
    if (t == 8 || t == 9 || t == 10 || t == 16)
      Throw(LFG_UNSUPPORTED, "Gmsh element type " + std::to_string(t) +
                                 " is a second-order (curved) element; this path carries TriaO1 / QuadO1 "
                                 "geometry only");
    int32_t v[4] = {-1, -1, -1, -1};
    for (int k = 0; k < MainNodesOf(t); ++k) {
      const int64_t mi = tag2mi[f.el_nodes[ee + k] - min_tag];
      if (mi < 0)
        Throw(LFG_IO_ERROR, "element " + std::to_string(e) + " references a node that is not a cell corner");
      v[k] = static_cast<int32_t>(mi);
    }
    if (t == 1) {
      g.edges.push_back(v[0]);
      g.edges.push_back(v[1]);
    } else {
      for (int k = 0; k < 4; ++k) g.cells.push_back(v[k]);
    }
    src[codim].push_back({e});
  }
  // physical numbers per entity
  for (int c = 0; c < 3; ++c) {
    g.phys_off[c].assign(1, 0);
    for (const auto& list : src[c]) {
      for (int64_t e : list) {
        if (f.version == 2) {
          g.phys_nr[c].push_back(f.el_phys[e]);
        } else {
          const auto& blk = f.blocks[f.el_block[e]];
          const auto& table = f.num_partitions > 0 ? f.part_entity_phys : f.entity_phys;
          auto it = table.find(blk);
          if (it != table.end())
            g.phys_nr[c].insert(g.phys_nr[c].end(), it->second.begin(), it->second.end());
        }
      }
      g.phys_off[c].push_back(static_cast<int64_t>(g.phys_nr[c].size()));
    }
  }
  for (const auto& pn : f.names) {
    const int codim = 2 - pn.dim;
    g.name2nr.insert({pn.name, {pn.nr, codim}});
    g.nr2name.insert({pn.nr, {pn.name, codim}});
  }
}

template <class F>
lfg_status Guard(F&& fn) {
  try {
    fn();
  } catch (const GmshError& e) {
    g_gmsh_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    g_gmsh_error = "host allocation failed";
    return LFG_OUT_OF_MEMORY;
  }
  g_gmsh_error.clear();
  return LFG_OK;
}

}  // namespace

extern "C" {

const char* lfg_gmsh_last_error(void) { return g_gmsh_error.c_str(); }

lfg_status lfg_gmsh_open_buffer(const char* data, int64_t size, lfg_gmsh** out) {
  if (!data || size < 0 || !out) return LFG_INVALID_ARG;
  *out = nullptr;
  return Guard([&] {
    auto* g = new lfg_gmsh;
    try {
      g->file = Parse(data, static_cast<size_t>(size), "<buffer>");
      Build(*g);
    } catch (...) {
      delete g;
      throw;
    }
    *out = g;
  });
}

lfg_status lfg_gmsh_open(const char* filename, lfg_gmsh** out) {
  if (!filename || !out) return LFG_INVALID_ARG;
  *out = nullptr;
  return Guard([&] {
    FILE* fp = std::fopen(filename, "rb");
    if (!fp) Throw(LFG_IO_ERROR, std::string("Could not open file ") + filename);
    std::string buf;
    std::fseek(fp, 0, SEEK_END);
    const long sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    if (sz < 0) {
      std::fclose(fp);
      Throw(LFG_IO_ERROR, std::string("Could not read file ") + filename);
    }
    buf.resize(static_cast<size_t>(sz));
    const size_t got = sz ? std::fread(&buf[0], 1, buf.size(), fp) : 0;
    std::fclose(fp);
    if (got != buf.size()) Throw(LFG_IO_ERROR, std::string("Could not read file ") + filename);
    auto* g = new lfg_gmsh;
    try {
      g->file = Parse(buf.data(), buf.size(), filename);
      Build(*g);
    } catch (...) {
      delete g;
      throw;
    }
    *out = g;
  });
}

lfg_status lfg_gmsh_destroy(lfg_gmsh* g) {
  delete g;
  return LFG_OK;
}

lfg_status lfg_gmsh_sizes(const lfg_gmsh* g, int64_t* num_nodes, int64_t* num_cells, int64_t* num_preset_edges) {
  if (!g) return LFG_INVALID_ARG;
  if (num_nodes) *num_nodes = static_cast<int64_t>(g->xy.size() / 2);
  if (num_cells) *num_cells = static_cast<int64_t>(g->cells.size() / 4);
  if (num_preset_edges) *num_preset_edges = static_cast<int64_t>(g->edges.size() / 2);
  return LFG_OK;
}

lfg_status lfg_gmsh_factory_input(const lfg_gmsh* g, double* xy, int32_t* cells, int32_t* preset_edges) {
  if (!g) return LFG_INVALID_ARG;
  if (xy) std::memcpy(xy, g->xy.data(), g->xy.size() * sizeof(double));
  if (cells) std::memcpy(cells, g->cells.data(), g->cells.size() * sizeof(int32_t));
  if (preset_edges && !g->edges.empty())
    std::memcpy(preset_edges, g->edges.data(), g->edges.size() * sizeof(int32_t));
  return LFG_OK;
}

lfg_status lfg_gmsh_build_mesh(lfg_ctx* ctx, const lfg_gmsh* g, lfg_mesh** mesh) {
  if (!ctx || !g || !mesh) return LFG_INVALID_ARG;
  return lfg_mesh_create(ctx, static_cast<int64_t>(g->xy.size() / 2), g->xy.data(),
                         static_cast<int64_t>(g->cells.size() / 4), g->cells.data(),
                         static_cast<int64_t>(g->edges.size() / 2), g->edges.empty() ? nullptr : g->edges.data(),
                         mesh);
}

lfg_status lfg_gmsh_physical_entity_nrs(const lfg_gmsh* g, int32_t codim, int64_t num_entities, int64_t* offsets,
                                        int32_t* nrs) {
  if (!g || codim < 0 || codim > 2 || num_entities < 0 || !offsets) return LFG_INVALID_ARG;
  const auto& off = g->phys_off[codim];
  const int64_t listed = static_cast<int64_t>(off.size()) - 1;
  for (int64_t i = 0; i <= num_entities; ++i) offsets[i] = off[std::min(i, listed)];
  if (nrs) {
    const int64_t n = offsets[num_entities];
    std::memcpy(nrs, g->phys_nr[codim].data(), static_cast<size_t>(n) * sizeof(int32_t));
  }
  return LFG_OK;
}

lfg_status lfg_gmsh_is_physical_entity(const lfg_gmsh* g, int32_t codim, int32_t nr, int64_t num_entities,
                                       uint8_t* flags) {
  if (!g || codim < 0 || codim > 2 || num_entities < 0 || !flags) return LFG_INVALID_ARG;
  const auto& off = g->phys_off[codim];
  const int64_t listed = static_cast<int64_t>(off.size()) - 1;
  for (int64_t i = 0; i < num_entities; ++i) {
    uint8_t hit = 0;
    if (i < listed)
      for (int64_t k = off[i]; k < off[i + 1]; ++k) hit |= g->phys_nr[codim][k] == nr;
    flags[i] = hit;
  }
  return LFG_OK;
}

// PhysicalEntityName2Nr (gmsh_reader.cc:32-66); codim -1: any.
lfg_status lfg_gmsh_name_to_nr(const lfg_gmsh* g, const char* name, int32_t codim, int32_t* nr) {
  if (!g || !name || !nr) return LFG_INVALID_ARG;
  return Guard([&] {
    auto range = g->name2nr.equal_range(name);
    if (range.first == range.second) Throw(LFG_NOT_FOUND, "No Physical Entity with this name found.");
    auto first = range.first;
    if (std::next(first) == range.second) {
      if (codim == -1 || codim == first->second.second) {
        *nr = first->second.first;
        return;
      }
    } else {
      if (codim == -1)
        Throw(LFG_NOT_FOUND, std::string("There are multiple physical entities with the name ") + name +
                                 ", please specify also the codimension.");
      for (auto it = first; it != range.second; ++it)
        if (it->second.second == codim) {
          *nr = it->second.first;
          return;
        }
    }
    Throw(LFG_NOT_FOUND, std::string("Physical Entity with name='") + name + "' and codimension=" +
                             std::to_string(codim) + "' not found.");
  });
}

// PhysicalEntityNr2Name (gmsh_reader.cc:68-99); codim -1: any.  The name is
// copied with its terminating zero into name (capacity bytes).
lfg_status lfg_gmsh_nr_to_name(const lfg_gmsh* g, int32_t nr, int32_t codim, char* name, int64_t capacity) {
  if (!g || !name || capacity <= 0) return LFG_INVALID_ARG;
  return Guard([&] {
    auto range = g->nr2name.equal_range(nr);
    if (range.first == range.second)
      Throw(LFG_NOT_FOUND, "Physical entity with number " + std::to_string(nr) + " not found.");
    const std::string* hit = nullptr;
    if (std::next(range.first) == range.second) {
      if (codim == -1 || codim == range.first->second.second) hit = &range.first->second.first;
    } else {
      if (codim == -1)
        Throw(LFG_NOT_FOUND, "There are multiple physical entities with the Number " + std::to_string(nr) +
                                 ", please specify also the codimension");
      for (auto it = range.first; it != range.second; ++it)
        if (it->second.second == codim) {
          hit = &it->second.first;
          break;
        }
    }
    if (!hit)
      Throw(LFG_NOT_FOUND, "Physical entity with number=" + std::to_string(nr) + ", codim=" +
                               std::to_string(codim) + " not found.");
    if (static_cast<int64_t>(hit->size()) + 1 > capacity) Throw(LFG_CAPACITY, "name buffer too small");
    std::memcpy(name, hit->c_str(), hit->size() + 1);
  });
}

// PhysicalEntities(codim) (gmsh_reader.cc:101-110): numbers in ascending
// order (count first; nrs may be NULL).
lfg_status lfg_gmsh_physical_entities(const lfg_gmsh* g, int32_t codim, int32_t* count, int32_t* nrs) {
  if (!g || !count) return LFG_INVALID_ARG;
  int32_t n = 0;
  for (const auto& p : g->nr2name)
    if (p.second.second == codim) {
      if (nrs) nrs[n] = p.first;
      ++n;
    }
  *count = n;
  return LFG_OK;
}

}  // extern "C"
