// fim_io.cpp -- the reference's file formats behind the C ABI:
//  * legacy ASCII VTK read/write, byte-compatible with load_vtk / save_vtk
//    (src/io/vtk.cpp:11-211), including its non-standard section order
//    (CELL_TYPES before CELLS), "%.3f" float points and INF written as -1;
//  * partition tags (read_vector_txt, src/io/io_base.h:81-86);
//  * the positional default.cfg (load_options, src/io/io_json.cpp:228-296)
//    and the JSON plan (load_plan / read_sim_from_json / read_funcs_from_json,
//    src/io/io_json.cpp:82-223, 299-317), with a small JSON reader of our own.
#include "../../include/fim.h"
#include "fim_internal.h"

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace {

int io_err(int code, const std::string &msg)
{
  fimgb::set_last_error(msg.c_str());
  return code;
}

// ---------------------------------------------------------------------------
// minimal JSON value + parser (objects keep keys sorted, as the reference's
// JSON library does by default, so iteration order matches)
struct JVal {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<JVal> arr;
  std::map<std::string, JVal> obj;
  const JVal *get(const std::string &k) const
  {
    if (kind != OBJ) return nullptr;
    auto it = obj.find(k);
    return it == obj.end() ? nullptr : &it->second;
  }
};

struct JParser {
  const char *p, *end;
  std::string err;
  void ws() { while (p < end && std::isspace((unsigned char)*p)) ++p; }
  bool fail(const char *m) { if (err.empty()) err = m; return false; }
  bool parse(JVal &v)
  {
    ws();
    if (p >= end) return fail("unexpected end of JSON");
    const char c = *p;
    if (c == '{') {
      ++p; v.kind = JVal::OBJ; ws();
      if (p < end && *p == '}') { ++p; return true; }
      for (;;) {
        ws();
        JVal key;
        if (p >= end || *p != '"' || !parse_str(key.str)) return fail("expected object key");
        ws();
        if (p >= end || *p != ':') return fail("expected ':'");
        ++p;
        JVal val;
        if (!parse(val)) return false;
        v.obj[key.str] = std::move(val);
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == '}') { ++p; return true; }
        return fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      ++p; v.kind = JVal::ARR; ws();
      if (p < end && *p == ']') { ++p; return true; }
      for (;;) {
        JVal val;
        if (!parse(val)) return false;
        v.arr.push_back(std::move(val));
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == ']') { ++p; return true; }
        return fail("expected ',' or ']'");
      }
    }
    if (c == '"') { v.kind = JVal::STR; return parse_str(v.str); }
    if (!std::strncmp(p, "true", 4)) { p += 4; v.kind = JVal::BOOL; v.b = true; return true; }
    if (!std::strncmp(p, "false", 5)) { p += 5; v.kind = JVal::BOOL; v.b = false; return true; }
    if (!std::strncmp(p, "null", 4)) { p += 4; v.kind = JVal::NUL; return true; }
    char *q = nullptr;
    v.num = std::strtod(p, &q);
    if (q == p) return fail("invalid JSON value");
    p = q;
    v.kind = JVal::NUM;
    return true;
  }
  bool parse_str(std::string &out)
  {
    ++p;  // opening quote
    while (p < end && *p != '"') {
      if (*p == '\\' && p + 1 < end) {
        ++p;
        switch (*p) {
          case 'n': out.push_back('\n'); break;
          case 't': out.push_back('\t'); break;
          case 'r': out.push_back('\r'); break;
          case 'b': out.push_back('\b'); break;
          case 'f': out.push_back('\f'); break;
          case 'u': out.push_back('?'); p += 4; break;
          default: out.push_back(*p);
        }
        ++p;
      } else {
        out.push_back(*p++);
      }
    }
    if (p >= end) return fail("unterminated string");
    ++p;
    return true;
  }
};

bool read_file(const char *path, std::string &out)
{
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::stringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

double num_of(const JVal *v, bool &ok)
{
  if (!v) { ok = false; return 0.0; }
  if (v->kind == JVal::NUM) return v->num;
  if (v->kind == JVal::BOOL) return v->b ? 1.0 : 0.0;
  ok = false;
  return 0.0;
}

}  // namespace

// ---------------------------------------------------------------------------
// VTK

extern "C" int fim_vtk_read(const char *path, int64_t *nV, int64_t *nT, double *xyz, int64_t *tets,
                            int32_t *etags)
{
  if (!path || !nV || !nT) return io_err(FIM_ERR_INVALID_ARGUMENT, "fim_vtk_read: NULL argument");
  std::ifstream f(path);
  if (!f) return io_err(FIM_ERR_IO, std::string("fim_vtk_read: cannot open ") + path);
  const bool fill = xyz != nullptr;
  std::string line;
  for (int i = 0; i < 4; ++i)  // version, title, format, dataset
    if (!std::getline(f, line)) return io_err(FIM_ERR_IO, "fim_vtk_read: truncated header");
  int64_t np = -1, nc = -1;
  while (std::getline(f, line)) {
    const size_t sp = line.find(' ');
    const std::string key = line.substr(0, sp);
    if (key == "POINTS") {
      np = std::atoll(line.c_str() + sp);
      if (np < 0) return io_err(FIM_ERR_IO, "fim_vtk_read: bad POINTS count");
      for (int64_t i = 0; i < np; ++i) {
        if (!std::getline(f, line)) return io_err(FIM_ERR_IO, "fim_vtk_read: truncated POINTS");
        if (fill) {
          if (std::sscanf(line.c_str(), "%lf %lf %lf", xyz + 3 * i, xyz + 3 * i + 1, xyz + 3 * i + 2) != 3)
            return io_err(FIM_ERR_IO, "fim_vtk_read: bad point line " + std::to_string(i));
        }
      }
    } else if (key == "CELLS") {
      nc = std::atoll(line.c_str() + sp);
      if (nc < 0) return io_err(FIM_ERR_IO, "fim_vtk_read: bad CELLS count");
      for (int64_t e = 0; e < nc; ++e) {
        if (!std::getline(f, line)) return io_err(FIM_ERR_IO, "fim_vtk_read: truncated CELLS");
        long long cnt = 0, a = 0, b = 0, c = 0, d = 0;
        const int k = std::sscanf(line.c_str(), "%lld %lld %lld %lld %lld", &cnt, &a, &b, &c, &d);
        if (k != 5 || cnt != 4) return io_err(FIM_ERR_IO, "fim_vtk_read: cell " + std::to_string(e) + " is not a tetrahedron");
        if (fill && tets) { tets[4 * e] = a; tets[4 * e + 1] = b; tets[4 * e + 2] = c; tets[4 * e + 3] = d; }
      }
    } else if (key == "CELL_TYPES") {
      const int64_t n = std::atoll(line.c_str() + sp);
      for (int64_t e = 0; e < n; ++e)
        if (!std::getline(f, line)) return io_err(FIM_ERR_IO, "fim_vtk_read: truncated CELL_TYPES");
    } else if (key == "CELL_DATA") {
      const int64_t n = std::atoll(line.c_str() + sp);
      std::getline(f, line);  // SCALARS
      std::getline(f, line);  // LOOKUP_TABLE
      for (int64_t e = 0; e < n; ++e) {
        if (!std::getline(f, line)) return io_err(FIM_ERR_IO, "fim_vtk_read: truncated CELL_DATA");
        if (fill && etags && e < nc) etags[e] = (int32_t)std::atoi(line.c_str());
      }
    }
  }
  if (np < 0 || nc < 0) return io_err(FIM_ERR_IO, "fim_vtk_read: no POINTS or CELLS section");
  *nV = np;
  *nT = nc;
  return FIM_OK;
}

extern "C" int fim_vtk_write(const char *path, int64_t nV, int64_t nT, const double *xyz, const int64_t *tets,
                             const int32_t *etags, const double *phi, const double *states)
{
  if (!path || !xyz || !tets || nV <= 0 || nT <= 0) return io_err(FIM_ERR_INVALID_ARGUMENT, "fim_vtk_write: bad argument");
  FILE *f = std::fopen(path, "w");
  if (!f) return io_err(FIM_ERR_IO, std::string("fim_vtk_write: cannot open ") + path);
  // the number of points written is the largest referenced id + 1 (vtk.cpp:118)
  int64_t maxid = -1;
  for (int64_t i = 0; i < 4 * nT; ++i) if (tets[i] > maxid) maxid = tets[i];
  const int numnodes = (int)(maxid + 1);
  const int numelems = (int)nT;
  (void)nV;
  std::fprintf(f, "# vtk DataFile Version 3.0\n");
  std::fprintf(f, "vtk output\n");
  std::fprintf(f, "ASCII\n");
  std::fprintf(f, "DATASET UNSTRUCTURED_GRID\n\n");
  std::fprintf(f, "POINTS %d     float\n", numnodes);
  for (int i = 0; i < numnodes; ++i) {
    const float x = (float)xyz[3 * i], y = (float)xyz[3 * i + 1], z = (float)xyz[3 * i + 2];
    std::fprintf(f, "%.3f %.3f %.3f\n", x, y, z);
  }
  std::fprintf(f, "CELL_TYPES %d\n", numelems);
  for (int i = 0; i < numelems; ++i) std::fprintf(f, "%d\n", 10);
  std::fprintf(f, "CELLS %d %lu\n", numelems, (unsigned long)(5 * (size_t)numelems));
  for (int i = 0; i < numelems; ++i)
    std::fprintf(f, "%d %ld %ld %ld %ld\n", 4, (long)tets[4 * i], (long)tets[4 * i + 1], (long)tets[4 * i + 2],
                 (long)tets[4 * i + 3]);
  std::fprintf(f, "CELL_DATA %d \n", numelems);
  std::fprintf(f, "SCALARS %s int %d\n", "elemTag", 1);
  std::fprintf(f, "LOOKUP_TABLE default\n");
  for (int i = 0; i < numelems; ++i) std::fprintf(f, "%d \n", etags ? etags[i] : 0);
  const double *data[2] = {phi, states};
  const char *names[2] = {"phi", "states"};
  if (phi || states) {
    std::fprintf(f, "POINT_DATA %d \n", numnodes);
    for (int n = 0; n < 2; ++n) {
      if (!data[n]) continue;
      std::fprintf(f, "SCALARS %s double %d\n", names[n], 1);
      std::fprintf(f, "LOOKUP_TABLE default\n");
      for (int i = 0; i < numnodes; ++i) std::fprintf(f, "%lf \n", (data[n][i] < 1e50) ? data[n][i] : -1);
    }
  }
  const int rc = std::ferror(f);
  std::fclose(f);
  return rc ? io_err(FIM_ERR_IO, "fim_vtk_write: write error") : FIM_OK;
}

extern "C" int fim_read_tags(const char *path, int64_t *n, int32_t *tags)
{
  if (!path || !n) return io_err(FIM_ERR_INVALID_ARGUMENT, "fim_read_tags: NULL argument");
  std::ifstream f(path);
  if (!f) return io_err(FIM_ERR_IO, std::string("fim_read_tags: cannot open ") + path);
  int64_t k = 0;
  long long v;
  while (f >> v) {
    if (tags) {
      if (k >= *n) return io_err(FIM_ERR_INVALID_ARGUMENT, "fim_read_tags: more tags than the given size");
      tags[k] = (int32_t)v;
    }
    ++k;
  }
  if (!f.eof()) return io_err(FIM_ERR_IO, "fim_read_tags: non-integer entry");
  *n = k;
  return FIM_OK;
}

// ---------------------------------------------------------------------------
// cfg + plan

extern "C" int fim_load_plan(const char *cfg_path, const char *plan_path, fim_plan_info *info, int64_t *stim)
{
  if (!info) return io_err(FIM_ERR_INVALID_ARGUMENT, "fim_load_plan: NULL info");
  const int64_t cap = stim ? info->n_stim_vertices : 0;
  std::memset(info, 0, sizeof(*info));
  // positional config: line 0 verbose, 2 solve type, 4 reentry flag, 7 dt, 8 n_steps
  if (cfg_path) {
    std::string txt;
    if (!read_file(cfg_path, txt)) return io_err(FIM_ERR_IO, std::string("fim_load_plan: cannot open ") + cfg_path);
    std::vector<std::string> lines;
    size_t pos = 0;
    while (pos <= txt.size()) {
      const size_t nl = txt.find('\n', pos);
      lines.push_back(txt.substr(pos, nl == std::string::npos ? std::string::npos : nl - pos));
      if (nl == std::string::npos) break;
      pos = nl + 1;
    }
    if (lines.size() < 9) return io_err(FIM_ERR_IO, "fim_load_plan: config has fewer than 9 lines");
    if (lines[0] != "false" && lines[0] != "true") return io_err(FIM_ERR_IO, "fim_load_plan: invalid value for verbose");
    if (lines[2] != "lin" && lines[2] != "vol") return io_err(FIM_ERR_IO, "fim_load_plan: invalid value for slvtype");
    if (lines[4] != "false" && lines[4] != "true") return io_err(FIM_ERR_IO, "fim_load_plan: invalid value for re_flag");
    char *q = nullptr;
    info->dt = std::strtod(lines[7].c_str(), &q) * 1000;
    if (*q) return io_err(FIM_ERR_IO, "fim_load_plan: invalid value for dt");
    info->n_steps = std::strtol(lines[8].c_str(), &q, 10);
    if (*q) return io_err(FIM_ERR_IO, "fim_load_plan: invalid value for t_max");
  }
  if (!plan_path) return FIM_OK;
  std::string txt;
  if (!read_file(plan_path, txt)) return io_err(FIM_ERR_IO, std::string("fim_load_plan: cannot open ") + plan_path);
  JVal root;
  JParser jp{txt.data(), txt.data() + txt.size(), {}};
  if (!jp.parse(root) || root.kind != JVal::OBJ) return io_err(FIM_ERR_IO, "fim_load_plan: JSON error: " + jp.err);

  // config -> function ids (sorted) -> first active region's CVref
  std::map<std::string, int> funcs;
  if (const JVal *cfg = root.get("config")) {
    for (const auto &kv : cfg->obj)
      if (const JVal *fn = kv.second.get("func"))
        if (fn->kind == JVal::STR) funcs[fn->str] = 1;
  }
  if (const JVal *fns = root.get("functions")) {
    for (const auto &kv : funcs) {
      const JVal *fn = fns->get(kv.first);
      if (!fn) continue;
      const JVal *ep = fn->get("EP");
      if (!ep || (ep->kind == JVal::OBJ && ep->obj.empty())) continue;  // inactive region
      const JVal *cv = fn->get("CV");
      const JVal *ref = cv ? cv->get("CVref") : nullptr;
      bool ok = true;
      const double vf = num_of(ref ? ref->get("vf") : nullptr, ok);
      const double vs = num_of(ref ? ref->get("vs") : nullptr, ok);
      const double vn = num_of(ref ? ref->get("vn") : nullptr, ok);
      if (ok && !info->has_cv) { info->cv[0] = vf; info->cv[1] = vs; info->cv[2] = vn; info->has_cv = 1; }
    }
  }
  const JVal *sim = root.get("simulation");
  if (!sim) return io_err(FIM_ERR_IO, "fim_load_plan: no simulation section");
  bool ok = true;
  const double dt = num_of(sim->get("deltatime"), ok);
  const double ns = num_of(sim->get("timesteps"), ok);
  if (!ok) return io_err(FIM_ERR_IO, "fim_load_plan: simulation.deltatime/timesteps missing");
  info->dt = dt * 1000.;
  info->n_steps = (int64_t)ns;
  const JVal *stims = sim->get("stimuli");
  int64_t nv = 0, nev = 0;
  bool first = true;
  if (stims && stims->kind == JVal::OBJ) {
    for (const auto &kv : stims->obj) {
      const JVal &s = kv.second;
      bool ok2 = true;
      const int active = (int)num_of(s.get("active"), ok2);
      const JVal *type = s.get("type");
      if (!ok2) return io_err(FIM_ERR_IO, "fim_load_plan: stimulus without 'active'");
      if (!active) continue;
      if (!type || type->kind != JVal::STR ||
          (type->str != "Transmembrane Current" && type->str != "Transmembrane Voltage clamp"))
        return io_err(FIM_ERR_IO, "fim_load_plan: unknown stim type");
      const JVal *prot = s.get("protocol");
      const double start = num_of(prot ? prot->get("start") : nullptr, ok2) * 1000.;
      const double npls = num_of(prot ? prot->get("npls") : nullptr, ok2);
      if (!ok2) return io_err(FIM_ERR_IO, "fim_load_plan: incomplete stimulus protocol");
      const JVal *el = s.get("electrode");
      const JVal *et = el ? el->get("type") : nullptr;
      std::vector<int64_t> vtx;
      if (et && et->kind == JVal::STR && et->str == "vtxdata") {
        const JVal *vd = el->get("vtxdata");
        if (vd && vd->kind == JVal::ARR)
          for (const auto &x : vd->arr) vtx.push_back((int64_t)x.num);
      }
      const int64_t reps = npls < 1 ? 1 : (int64_t)npls;
      for (int64_t r = 0; r < reps; ++r) {
        for (int64_t x : vtx) {
          if (stim && nv < cap) stim[nv] = x;
          ++nv;
        }
        ++nev;
      }
      if (first) { info->tstart = start; first = false; }
    }
  }
  info->n_events = nev;
  info->n_stim_vertices = nv;
  if (stim && nv > cap) return io_err(FIM_ERR_INVALID_ARGUMENT, "fim_load_plan: stimulus buffer too small");
  return FIM_OK;
}
