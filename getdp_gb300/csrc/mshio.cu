// Gmsh MSH 2.2 reader (ASCII and binary), host code: the mesh GetDP reads
// with Geo_ReadFileWithGmsh (GeoData.cpp) parsed at memory speed, for the
// element tables of the batched Generate.  Elements are kept grouped by
// Gmsh type in file order; node references stay Gmsh node numbers.
#include <cerrno>
#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

struct gb300_msh {
  struct Group {
    int type = 0, ntags = 0, npe = 0;
    std::vector<long long> num;    // element numbers
    std::vector<int> tags;         // count x ntags
    std::vector<long long> nodes;  // count x npe (Gmsh node numbers)
  };
  std::vector<long long> node_num;
  std::vector<double> xyz;
  std::vector<Group> groups;
};

namespace {

int nodes_of_type(int t)
{
  switch(t) {
  case 1: return 2;   // line
  case 2: return 3;   // triangle
  case 3: return 4;   // quadrangle
  case 4: return 4;   // tetrahedron
  case 5: return 8;   // hexahedron
  case 6: return 6;   // prism
  case 7: return 5;   // pyramid
  case 8: return 3;   // second-order line
  case 9: return 6;   // second-order triangle
  case 11: return 10; // second-order tetrahedron
  case 15: return 1;  // point
  default: return -1;
  }
}

struct Cursor {
  const char *p, *end;
  bool ok = true;
  void skip()
  {
    while(p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
  }
  long long integer()
  {
    skip();
    bool neg = false;
    if(p < end && (*p == '-' || *p == '+')) neg = (*p++ == '-');
    if(p >= end || *p < '0' || *p > '9') {
      ok = false;
      return 0;
    }
    long long v = 0;
    while(p < end && *p >= '0' && *p <= '9') v = v * 10 + (*p++ - '0');
    return neg ? -v : v;
  }
  double real()
  {
    // bounded by the buffer's end and correctly rounded, like strtod on a
    // terminated string (std::from_chars takes no leading '+')
    skip();
    if(p < end && *p == '+') p++;
    double v = 0.;
    auto r = std::from_chars(p, end, v);
    if(r.ec != std::errc() || r.ptr == p) {
      ok = false;
      return 0.;
    }
    p = r.ptr;
    return v;
  }
  bool line_starting(const char *tag)
  {
    // advance to the line that starts with tag, then past it
    size_t n = strlen(tag);
    while(p < end) {
      if((size_t)(end - p) >= n && !memcmp(p, tag, n)) {
        p += n;
        while(p < end && *p != '\n') p++;
        if(p < end) p++;
        return true;
      }
      while(p < end && *p != '\n') p++;
      if(p < end) p++;
    }
    return false;
  }
};

gb300_msh::Group &group_for(gb300_msh &m, int type, int ntags)
{
  for(auto &g : m.groups)
    if(g.type == type && g.ntags == ntags) return g;
  m.groups.emplace_back();
  auto &g = m.groups.back();
  g.type = type;
  g.ntags = ntags;
  g.npe = nodes_of_type(type);
  return g;
}

}  // namespace

extern "C" {

int gb300_msh_read(const char *path, gb300_msh **out)
{
  if(!path || !out) {
    gb::set_error("msh: null argument");
    return GB300_ERR_ARG;
  }
  FILE *f = fopen(path, "rb");
  if(!f) {
    gb::set_error("msh: cannot open '%s': %s", path, strerror(errno));
    return GB300_ERR_ARG;
  }
  fseek(f, 0, SEEK_END);
  long size = ftell(f);
  fseek(f, 0, SEEK_SET);
  std::string buf(size > 0 ? (size_t)size : 0, '\0');
  size_t got = size > 0 ? fread(&buf[0], 1, (size_t)size, f) : 0;
  fclose(f);
  if((long)got != size) {
    gb::set_error("msh: short read of '%s'", path);
    return GB300_ERR_ARG;
  }
  Cursor c{buf.data(), buf.data() + buf.size()};
  if(!c.line_starting("$MeshFormat")) {
    gb::set_error("msh: '%s' has no $MeshFormat", path);
    return GB300_ERR_ARG;
  }
  double version = c.real();
  int binary = (int)c.integer();
  int dsize = (int)c.integer();
  if(!c.ok || version < 2. || version >= 3. || dsize != 8) {
    gb::set_error("msh: '%s' is not MSH 2.x with 8-byte reals", path);
    return GB300_ERR_UNSUPPORTED;
  }
  if(binary) {  // the endianness marker: int 1
    c.p = strchr(c.p, '\n') + 1;
    int one = 0;
    memcpy(&one, c.p, 4);
    if(one != 1) {
      gb::set_error("msh: '%s' has another byte order", path);
      return GB300_ERR_UNSUPPORTED;
    }
  }
  gb300_msh *m = new gb300_msh();
  auto fail = [&](const char *what) {
    gb::set_error("msh: '%s': %s", path, what);
    delete m;
    return GB300_ERR_ARG;
  };
  if(!c.line_starting("$Nodes")) return fail("no $Nodes");
  long long nn = c.integer();
  if(!c.ok || nn < 0) return fail("bad node count");
  m->node_num.resize(nn);
  m->xyz.resize(3 * nn);
  if(binary) {
    c.p = strchr(c.p, '\n') + 1;
    if(c.end - c.p < nn * 28) return fail("truncated binary nodes");
    for(long long i = 0; i < nn; i++) {
      int num;
      memcpy(&num, c.p, 4);
      memcpy(&m->xyz[3 * i], c.p + 4, 24);
      m->node_num[i] = num;
      c.p += 28;
    }
  }
  else
    for(long long i = 0; i < nn; i++) {
      m->node_num[i] = c.integer();
      m->xyz[3 * i] = c.real();
      m->xyz[3 * i + 1] = c.real();
      m->xyz[3 * i + 2] = c.real();
    }
  if(!c.ok) return fail("bad node record");
  if(!c.line_starting("$Elements")) return fail("no $Elements");
  long long ne = c.integer();
  if(!c.ok || ne < 0) return fail("bad element count");
  if(binary) {
    c.p = strchr(c.p, '\n') + 1;
    long long done = 0;
    while(done < ne) {
      if(c.end - c.p < 12) return fail("truncated binary elements");
      int hdr[3];
      memcpy(hdr, c.p, 12);
      c.p += 12;
      int npe = nodes_of_type(hdr[0]);
      if(npe < 0 || hdr[1] <= 0 || hdr[2] < 0) return fail("unsupported element type");
      auto &g = group_for(*m, hdr[0], hdr[2]);
      long long rl = 1 + hdr[2] + npe;
      if(c.end - c.p < (long long)hdr[1] * rl * 4) return fail("truncated binary elements");
      std::vector<int> rec(rl);
      for(int k = 0; k < hdr[1]; k++) {
        memcpy(rec.data(), c.p, 4 * rl);
        c.p += 4 * rl;
        g.num.push_back(rec[0]);
        for(int t = 0; t < hdr[2]; t++) g.tags.push_back(rec[1 + t]);
        for(int v = 0; v < npe; v++) g.nodes.push_back(rec[1 + hdr[2] + v]);
      }
      done += hdr[1];
    }
  }
  else
    for(long long k = 0; k < ne; k++) {
      long long num = c.integer();
      int type = (int)c.integer();
      int ntags = (int)c.integer();
      int npe = nodes_of_type(type);
      if(!c.ok || npe < 0 || ntags < 0) return fail("unsupported element record");
      auto &g = group_for(*m, type, ntags);
      g.num.push_back(num);
      for(int t = 0; t < ntags; t++) g.tags.push_back((int)c.integer());
      for(int v = 0; v < npe; v++) g.nodes.push_back(c.integer());
    }
  if(!c.ok) return fail("bad element record");
  *out = m;
  return GB300_OK;
}

int gb300_msh_free(gb300_msh *m)
{
  delete m;
  return GB300_OK;
}

int gb300_msh_nodes(const gb300_msh *m, long long *n, const long long **numbers,
                    const double **xyz)
{
  if(!m || !n || !numbers || !xyz) {
    gb::set_error("msh: null argument");
    return GB300_ERR_ARG;
  }
  *n = (long long)m->node_num.size();
  *numbers = m->node_num.data();
  *xyz = m->xyz.data();
  return GB300_OK;
}

int gb300_msh_group_count(const gb300_msh *m, int *count)
{
  if(!m || !count) {
    gb::set_error("msh: null argument");
    return GB300_ERR_ARG;
  }
  *count = (int)m->groups.size();
  return GB300_OK;
}

int gb300_msh_group(const gb300_msh *m, int g, int *type, long long *n_elems,
                    int *n_tags, int *nodes_per_elem, const long long **numbers,
                    const int **tags, const long long **nodes)
{
  if(!m || g < 0 || g >= (int)m->groups.size() || !type || !n_elems || !n_tags ||
     !nodes_per_elem || !numbers || !tags || !nodes) {
    gb::set_error("msh: bad group query");
    return GB300_ERR_ARG;
  }
  const auto &G = m->groups[g];
  *type = G.type;
  *n_elems = (long long)G.num.size();
  *n_tags = G.ntags;
  *nodes_per_elem = G.npe;
  *numbers = G.num.data();
  *tags = G.tags.data();
  *nodes = G.nodes.data();
  return GB300_OK;
}

}  // extern "C"
