#include "fe_msh.h"

#include <algorithm>
#include <fstream>
#include <unordered_map>

#include "fe_common.h"

namespace feng {

std::string MshData::name_of(int dim, int tag) const
{
  auto ph = entityPhys.find({dim, tag});
  if(ph == entityPhys.end()) return "";
  auto nm = physNames.find({dim, ph->second});
  return nm == physNames.end() ? "" : nm->second;
}

int read_msh41(const std::string &path, MshData &out)
{
  std::ifstream in(path);
  if(!in.good()) {
    set_error("mesh file \"%s\" does not exist", path.c_str());
    return FE_READ_ERROR;
  }
  out = MshData();
  std::unordered_map<long long, int32_t> nodeIndex;  // gmsh node tag -> index
  std::string tok;
  while(in >> tok) {
    if(tok == "$MeshFormat") {
      double ver = 0; int ftype = -1, dsize;
      in >> ver >> ftype >> dsize;
      // the 4.1 layout only (4.0 lists node tags and coordinates differently)
      if(!in || ver < 4.1 - 1e-9 || ver >= 5.0 || ftype != 0) {
        set_error("only ASCII msh 4.1 is supported (got %g, type %d)", ver, ftype);
        return FE_READ_ERROR;
      }
    } else if(tok == "$PhysicalNames") {
      int np = 0; in >> np;
      for(int i = 0; i < np; ++i) {
        int d, t; std::string name;
        in >> d >> t;
        std::getline(in, name);
        if(!in) { set_error("truncated $PhysicalNames"); return FE_READ_ERROR; }
        size_t a = name.find('"'), b = name.rfind('"');
        if(a == std::string::npos || b <= a) { set_error("bad physical name"); return FE_READ_ERROR; }
        out.physNames[{d, t}] = name.substr(a + 1, b - a - 1);
      }
    } else if(tok == "$Entities") {
      int np = 0, nc = 0, ns = 0, nvol = 0; in >> np >> nc >> ns >> nvol;
      for(int i = 0; i < np; ++i) {
        int tag, nphys; double a, b, c; in >> tag >> a >> b >> c >> nphys;
        for(int j = 0; j < nphys; ++j) { int p; in >> p; if(j == 0) out.entityPhys[{0, tag}] = p; }
      }
      for(int d = 1; d <= 3; ++d) {
        int cnt = d == 1 ? nc : d == 2 ? ns : nvol;
        for(int i = 0; i < cnt; ++i) {
          int tag, nphys, nbnd; double bb[6];
          in >> tag;
          for(double &v : bb) in >> v;
          in >> nphys;
          for(int j = 0; j < nphys; ++j) { int p; in >> p; if(j == 0) out.entityPhys[{d, tag}] = p; }
          in >> nbnd;
          if(!in) { set_error("truncated $Entities"); return FE_READ_ERROR; }
          for(int j = 0; j < nbnd; ++j) { int q; in >> q; }
        }
      }
      if(!in) { set_error("truncated $Entities"); return FE_READ_ERROR; }
    } else if(tok == "$Nodes") {
      long long nblocks = 0, nnodes = -1, mn, mx; in >> nblocks >> nnodes >> mn >> mx;
      if(!in || nnodes < 0 || nnodes > (1ll << 31) - 1) { set_error("bad node count"); return FE_READ_ERROR; }
      out.x.resize(nnodes); out.y.resize(nnodes); out.z.resize(nnodes);
      int32_t cnt = 0;
      for(long long b = 0; b < nblocks; ++b) {
        int d, t, par; long long nn = -1; in >> d >> t >> par >> nn;
        if(!in || nn < 0 || cnt + nn > nnodes) { set_error("bad node block"); return FE_READ_ERROR; }
        std::vector<long long> tags(nn);
        for(auto &tg : tags) in >> tg;
        for(long long i = 0; i < nn; ++i) {
          double x, y, z; in >> x >> y >> z;
          if(!in) { set_error("truncated node block"); return FE_READ_ERROR; }
          nodeIndex[tags[i]] = cnt;
          out.x[cnt] = x; out.y[cnt] = y; out.z[cnt] = z; ++cnt;
        }
      }
      if(cnt != nnodes || (long long)nodeIndex.size() != nnodes) {
        set_error("vertex indices are not unique"); return FE_READ_ERROR;
      }
    } else if(tok == "$Elements") {
      long long nblocks = 0, nel, mn, mx; in >> nblocks >> nel >> mn >> mx;
      if(!in || nblocks < 0) { set_error("bad $Elements header"); return FE_READ_ERROR; }
      for(long long b = 0; b < nblocks; ++b) {
        MshBlock blk;
        long long ne = -1;
        in >> blk.dim >> blk.tag >> blk.type >> ne;
        if(!in) { set_error("truncated element block header"); return FE_READ_ERROR; }
        const int npe = blk.type == 15 ? 1 : blk.type == 1 ? 2 : blk.type == 2 ? 3 : blk.type == 4 ? 4 : -1;
        if(npe < 0) { set_error("unsupported gmsh element type %d", blk.type); return FE_READ_ERROR; }
        if(ne < 0) { set_error("bad element block"); return FE_READ_ERROR; }
        blk.nodes.reserve((size_t)std::min<long long>(ne, 1ll << 24) * npe);
        for(long long e = 0; e < ne; ++e) {
          long long etag; in >> etag;
          for(int k = 0; k < npe; ++k) {
            long long nt = 0; in >> nt;
            if(!in) { set_error("truncated element block"); return FE_READ_ERROR; }
            auto it = nodeIndex.find(nt);
            if(it == nodeIndex.end()) { set_error("element node %lld does not exist", nt); return FE_READ_ERROR; }
            blk.nodes.push_back(it->second);
          }
        }
        out.blocks.push_back(std::move(blk));
      }
    }
  }
  if(in.bad()) { set_error("read error on %s", path.c_str()); return FE_READ_ERROR; }
  return FE_OK;
}

}  // namespace feng
