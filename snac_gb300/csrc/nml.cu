// nml.cu -- the reference's input files, read on the host (param.f90:88-240).
//
// dns.nml holds the &dns, &scalar and &hypre groups, blocks.nml the &blocks group.  The reader
// understands the list-directed namelist forms these files use: "name = v1, v2, ..." for scalars and
// whole arrays, array sections "name(0:1,1:3,2,1) = ..." filled in Fortran (column-major) order, repeat
// counts "3*0.", quoted strings, logicals (T, F, .true., .false.), reals with d/D exponents, "!" comments
// and a closing "/".  Unset entries keep the reference's defaults (param.f90:108-133, 147-153, 166-167).
// Host code only: no device is needed.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "snac_internal.h"

namespace snac {
namespace {

struct Assign {
  std::vector<std::pair<int, int>> dims;  // (lower, upper) per subscript; lower == upper for a single index
  std::vector<std::string> values;        // tokens after expanding repeat counts
};
using Group = std::map<std::string, std::vector<Assign>>;

std::string lower(std::string s) {
  for (auto &ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

// split the text of one group into "name[(subscripts)] = values" assignments
bool parse_group(const std::string &text, const std::string &group, Group &out, std::string &err) {
  // strip comments outside quotes
  std::string t;
  bool inq = false;
  char qc = 0;
  for (size_t i = 0; i < text.size(); i++) {
    const char ch = text[i];
    if (inq) {
      t += ch;
      if (ch == qc) inq = false;
    } else if (ch == '\'' || ch == '"') {
      inq = true;
      qc = ch;
      t += ch;
    } else if (ch == '!') {
      while (i < text.size() && text[i] != '\n') i++;
      t += '\n';
    } else {
      t += ch;
    }
  }
  // find "&group"
  const std::string lt = lower(t);
  size_t p = 0;
  for (;;) {
    p = lt.find("&" + group, p);
    if (p == std::string::npos) return false;
    const size_t e = p + 1 + group.size();
    if (e >= lt.size() || !(std::isalnum((unsigned char)lt[e]) || lt[e] == '_')) break;
    p = e;
  }
  size_t i = p + 1 + group.size();
  // tokens until the terminating '/' (outside quotes)
  std::vector<std::string> toks;
  std::string cur;
  auto flush = [&]() {
    if (!cur.empty()) toks.push_back(cur);
    cur.clear();
  };
  bool done = false;
  for (; i < t.size() && !done; i++) {
    const char ch = t[i];
    if (ch == '\'' || ch == '"') {
      flush();
      const char q = ch;
      std::string s(1, q);
      for (i++; i < t.size() && t[i] != q; i++) s += t[i];
      s += q;
      toks.push_back(s);
    } else if (ch == '/' || ch == '&') {
      flush();
      done = true;
    } else if (ch == '=' || ch == ',') {
      flush();
      if (ch == '=') toks.push_back("=");
    } else if (ch == '(') {
      // subscripts belong to the name before them (also when blanks separate them)
      std::string s;
      for (; i < t.size() && t[i] != ')'; i++)
        if (!std::isspace((unsigned char)t[i])) s += t[i];
      if (cur.empty() && !toks.empty() && toks.back() != "=") {
        cur = toks.back();
        toks.pop_back();
      }
      cur += s + ")";
    } else if (std::isspace((unsigned char)ch)) {
      flush();
    } else {
      cur += ch;
    }
  }
  flush();
  // assignments: NAME = v v v NAME = ...
  size_t k = 0;
  while (k < toks.size()) {
    if (k + 1 >= toks.size() || toks[k + 1] != "=") { err = "namelist &" + group + ": cannot parse near '" + toks[k] + "'"; return true; }
    std::string name = lower(toks[k]);
    Assign a;
    const size_t lp = name.find('(');
    if (lp != std::string::npos) {
      const std::string sub = name.substr(lp + 1, name.size() - lp - 2);
      name = name.substr(0, lp);
      size_t s0 = 0;
      while (s0 <= sub.size()) {
        size_t s1 = sub.find(',', s0);
        if (s1 == std::string::npos) s1 = sub.size();
        const std::string d = sub.substr(s0, s1 - s0);
        const size_t c = d.find(':');
        if (c == std::string::npos) a.dims.push_back({std::atoi(d.c_str()), std::atoi(d.c_str())});
        else a.dims.push_back({std::atoi(d.substr(0, c).c_str()), std::atoi(d.substr(c + 1).c_str())});
        s0 = s1 + 1;
      }
    }
    k += 2;
    while (k < toks.size() && !(k + 1 < toks.size() && toks[k + 1] == "=")) {
      const std::string &v = toks[k];
      const size_t star = v.find('*');
      if (star != std::string::npos && v[0] != '\'' && v[0] != '"' && star > 0 &&
          std::isdigit((unsigned char)v[0])) {
        const int rep = std::atoi(v.substr(0, star).c_str());
        for (int r = 0; r < rep; r++) a.values.push_back(v.substr(star + 1));
      } else {
        a.values.push_back(v);
      }
      k++;
    }
    out[name].push_back(a);
  }
  return true;
}

double to_real(std::string v) {
  for (auto &ch : v)
    if (ch == 'd' || ch == 'D') ch = 'e';
  return std::strtod(v.c_str(), nullptr);
}
int to_int(const std::string &v) { return std::atoi(v.c_str()); }
bool to_logical(std::string v) {
  v = lower(v);
  size_t i = 0;
  while (i < v.size() && v[i] == '.') i++;
  return i < v.size() && v[i] == 't';
}
std::string to_string(const std::string &v) {
  if (v.size() >= 2 && (v[0] == '\'' || v[0] == '"')) return v.substr(1, v.size() - 2);
  return v;
}

// the flat (column-major) offsets an assignment covers, for an array with the given lower bounds and
// extents; a whole-array assignment covers the first values.size() elements
bool offsets(const Assign &a, const std::vector<int> &lb, const std::vector<int> &ext, std::vector<long> &off,
             std::string &err, const std::string &name) {
  off.clear();
  long total = 1;
  for (int e : ext) total *= e;
  if (a.dims.empty()) {
    for (size_t q = 0; q < a.values.size() && (long)q < total; q++) off.push_back((long)q);
    return true;
  }
  if (a.dims.size() != ext.size()) { err = name + ": wrong number of subscripts"; return false; }
  std::vector<int> idx(ext.size());
  for (size_t d = 0; d < ext.size(); d++) {
    if (a.dims[d].first < lb[d] || a.dims[d].second > lb[d] + ext[d] - 1 || a.dims[d].first > a.dims[d].second) {
      err = name + ": subscript out of range";
      return false;
    }
    idx[d] = a.dims[d].first;
  }
  for (;;) {
    long o = 0, st = 1;
    for (size_t d = 0; d < ext.size(); d++) { o += (idx[d] - lb[d]) * st; st *= ext[d]; }
    off.push_back(o);
    size_t d = 0;
    for (; d < ext.size(); d++) {
      if (++idx[d] <= a.dims[d].second) break;
      idx[d] = a.dims[d].first;
    }
    if (d == ext.size()) break;
  }
  return true;
}

template <typename F>
bool assign_all(const Group &g, const std::string &name, const std::vector<int> &lb, const std::vector<int> &ext,
                F set, std::string &err) {
  auto it = g.find(name);
  if (it == g.end()) return true;
  for (const Assign &a : it->second) {
    std::vector<long> off;
    if (!offsets(a, lb, ext, off, err, name)) return false;
    for (size_t q = 0; q < off.size() && q < a.values.size(); q++) set(off[q], a.values[q]);
  }
  return true;
}

bool read_file(const char *path, std::string &text) {
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return false;
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), fp)) > 0) text.append(buf, n);
  std::fclose(fp);
  return true;
}

}  // namespace
}  // namespace snac

using namespace snac;

int snac_read_namelists(const char *dns_path, const char *blocks_path, int fft_axis, int impdiff, int boussinesq,
                        snac_case *c, snac_block_desc *blocks, int max_blocks) {
  if (!dns_path || !blocks_path || !c || !blocks || max_blocks < 1) {
    set_error("snac_read_namelists: null argument");
    return SNAC_ERR_ARG;
  }
  std::string dns, blk, err;
  if (!read_file(dns_path, dns)) { set_error("cannot open %s", dns_path); return SNAC_ERR_IO; }
  if (!read_file(blocks_path, blk)) { set_error("cannot open %s", blocks_path); return SNAC_ERR_IO; }
  // defaults (param.f90:108-133); hypre_tol/maxiter defaults of param.f90:15-17 (the tolerance is the
  // single-precision literal 1.e-4 widened to FP64)
  std::memset(c, 0, sizeof(*c));
  c->visci = 1.0;
  c->dt_f = -1.0;
  c->tol = (double)1.e-4f;
  c->maxiter = 50;
  c->fft_axis = fft_axis;
  c->impdiff = impdiff;
  c->boussinesq = boussinesq;
  Group gd, gs, gh, gb;
  if (!parse_group(dns, "dns", gd, err)) { set_error("dns namelist not found in %s", dns_path); return SNAC_ERR_ARG; }
  if (!err.empty()) { set_error("%s", err.c_str()); return SNAC_ERR_ARG; }
  parse_group(dns, "hypre", gh, err);
  if (!err.empty()) { set_error("%s", err.c_str()); return SNAC_ERR_ARG; }
  const std::vector<int> one = {1}, three = {3};
  auto rd = [&](const Group &g, const char *n, double *dst, int cnt) {
    return assign_all(g, n, std::vector<int>{1}, std::vector<int>{cnt}, [&](long o, const std::string &v) { dst[o] = to_real(v); }, err);
  };
  auto ri = [&](const Group &g, const char *n, int *dst, int cnt) {
    return assign_all(g, n, std::vector<int>{1}, std::vector<int>{cnt}, [&](long o, const std::string &v) { dst[o] = to_int(v); }, err);
  };
  bool ok = rd(gd, "cfl", &c->cfl, 1) && rd(gd, "dtmax", &c->dtmax, 1) && rd(gd, "dt_f", &c->dt_f, 1) &&
            rd(gd, "visci", &c->visci, 1) && ri(gd, "icheck", &c->icheck, 1) && rd(gd, "bforce", c->bforce, 3) &&
            rd(gd, "gacc", c->gacc, 3) && ri(gd, "nscal", &c->nscal, 1) && rd(gh, "hypre_tol", &c->tol, 1) &&
            ri(gh, "hypre_maxiter", &c->maxiter, 1);
  if (!ok) { set_error("%s", err.c_str()); return SNAC_ERR_ARG; }
  if (c->nscal < 0) c->nscal = 0;
  if (c->nscal > SNAC_MAX_SCAL) { set_error("nscal > %d is not supported", SNAC_MAX_SCAL); return SNAC_ERR_UNSUPPORTED; }
  if (boussinesq && c->nscal == 0) { set_error("_BOUSSINESQ_BUOYANCY requires nscal > 0"); return SNAC_ERR_ARG; }
  const int ns = c->nscal;
  if (ns > 0) {  // param.f90:141-153
    for (int q = 0; q < ns; q++) { c->alphai[q] = 1.79769313486231570e308; c->ssource[q] = 0; c->scalf[q] = 0; c->is_sforced[q] = 0; }
    if (!parse_group(dns, "scalar", gs, err)) { set_error("scalar namelist not found in %s", dns_path); return SNAC_ERR_ARG; }
    ok = rd(gs, "alphai", c->alphai, ns) && rd(gs, "beta", &c->beta, 1) && rd(gs, "ssource", c->ssource, ns) &&
         rd(gs, "scalf", c->scalf, ns) &&
         assign_all(gs, "is_sforced", std::vector<int>{1}, std::vector<int>{ns},
                    [&](long o, const std::string &v) { c->is_sforced[o] = to_logical(v) ? 1 : 0; }, err);
    if (!ok) { set_error("%s", err.c_str()); return SNAC_ERR_ARG; }
  }
  // &blocks (param.f90:120-133 defaults)
  if (!parse_group(blk, "blocks", gb, err)) { set_error("blocks namelist not found in %s", blocks_path); return SNAC_ERR_ARG; }
  if (!err.empty()) { set_error("%s", err.c_str()); return SNAC_ERR_ARG; }
  int nb = 0;
  if (!ri(gb, "nblocks", &nb, 1)) { set_error("%s", err.c_str()); return SNAC_ERR_ARG; }
  if (nb < 1 || nb > max_blocks) { set_error("invalid number of blocks in blocks.nml (%d)", nb); return SNAC_ERR_ARG; }
  c->nblocks = nb;
  for (int b = 0; b < nb; b++) {
    snac_block_desc &B = blocks[b];
    std::memset(&B, 0, sizeof(B));
    for (int a = 0; a < 3; a++) {
      B.ng[a] = 1;
      B.lmin[a] = 0.0;
      B.lmax[a] = 1.0;
      for (int s = 0; s < 2; s++) {
        for (int v = 0; v < 3; v++) B.cbcvel[v][a][s] = 'D';
        B.cbcpre[a][s] = 'N';
        for (int q = 0; q < SNAC_MAX_SCAL; q++) B.cbcscal[q][a][s] = 'N';
      }
    }
  }
  const int mb = nb;
  // block_xxx(1:3, iblock)
  auto per_axis_i = [&](const char *n, int(snac_block_desc::*m)[3]) {
    return assign_all(gb, n, std::vector<int>{1, 1}, std::vector<int>{3, mb},
                      [&](long o, const std::string &v) { (blocks[o / 3].*m)[o % 3] = to_int(v); }, err);
  };
  auto per_axis_d = [&](const char *n, double(snac_block_desc::*m)[3]) {
    return assign_all(gb, n, std::vector<int>{1, 1}, std::vector<int>{3, mb},
                      [&](long o, const std::string &v) { (blocks[o / 3].*m)[o % 3] = to_real(v); }, err);
  };
  // block_cbcpre(0:1,1:3,iblock): side fastest, then direction
  auto face = [&](const char *n, auto setter) {
    return assign_all(gb, n, std::vector<int>{0, 1, 1}, std::vector<int>{2, 3, mb},
                      [&](long o, const std::string &v) { setter(blocks[o / 6], (int)(o % 6) / 2, (int)(o % 2), v); }, err);
  };
  // block_cbcvel(0:1,1:3,1:3,iblock): side, direction, component
  auto face_vel = [&](const char *n, auto setter) {
    return assign_all(gb, n, std::vector<int>{0, 1, 1, 1}, std::vector<int>{2, 3, 3, mb},
                      [&](long o, const std::string &v) {
                        setter(blocks[o / 18], (int)(o % 18) / 6, (int)(o % 6) / 2, (int)(o % 2), v);
                      }, err);
  };
  const int nsx = std::max(ns, 1);
  auto face_scal = [&](const char *n, auto setter) {
    return assign_all(gb, n, std::vector<int>{0, 1, 1, 1}, std::vector<int>{2, 3, nsx, mb},
                      [&](long o, const std::string &v) {
                        const long per = 6L * nsx;
                        setter(blocks[o / per], (int)((o % per) / 6), (int)(o % 6) / 2, (int)(o % 2), v);
                      }, err);
  };
  auto ch = [](const std::string &v) { const std::string s = to_string(v); return s.empty() ? ' ' : s[0]; };
  ok = per_axis_i("block_ng", &snac_block_desc::ng) && per_axis_d("block_lmin", &snac_block_desc::lmin) &&
       per_axis_d("block_lmax", &snac_block_desc::lmax) && per_axis_i("block_gt", &snac_block_desc::gt) &&
       per_axis_d("block_gr", &snac_block_desc::gr) &&
       face("block_cbcpre", [&](snac_block_desc &B, int a, int s, const std::string &v) { B.cbcpre[a][s] = ch(v); }) &&
       face("block_bcpre", [&](snac_block_desc &B, int a, int s, const std::string &v) { B.bcpre[a][s] = to_real(v); }) &&
       face("block_inflow_type",
            [&](snac_block_desc &B, int a, int s, const std::string &v) { B.inflow_type[a][s] = to_int(v); }) &&
       face_vel("block_cbcvel",
                [&](snac_block_desc &B, int comp, int a, int s, const std::string &v) { B.cbcvel[comp][a][s] = ch(v); }) &&
       face_vel("block_bcvel",
                [&](snac_block_desc &B, int comp, int a, int s, const std::string &v) { B.bcvel[comp][a][s] = to_real(v); }) &&
       face_scal("block_cbcscal",
                 [&](snac_block_desc &B, int q, int a, int s, const std::string &v) { if (q < SNAC_MAX_SCAL) B.cbcscal[q][a][s] = ch(v); }) &&
       face_scal("block_bcscal",
                 [&](snac_block_desc &B, int q, int a, int s, const std::string &v) { if (q < SNAC_MAX_SCAL) B.bcscal[q][a][s] = to_real(v); });
  if (!ok) { set_error("%s", err.c_str()); return SNAC_ERR_ARG; }
  // one task per block: block_dims other than 1 describe an MPI split that a single GPU does not need
  return SNAC_OK;
}
