// Output in the reference's formats (include/eqfield.h: eqf_json_*, eqf_vtk_*).
//
// Host code over the public C ABI.  The JSON recording follows jsonRecording
// (src/main.cpp:81-192, version v00_02) and streams each frame to the file as it is
// recorded; the VTK snapshots follow what DOLFIN's File writes for
// fenicsInterface::writeDiffusionFiles (src/fHSL.cpp:606-632): a .pvd collection and
// one .vtu per snapshot.  Doubles are written with the fewest digits that read back
// to the same value (integral values with a trailing ".0", non-finite ones as null,
// as the reference's JSON library does).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/eqfield.h"

namespace {

void put_double(std::string& o, double v) {
  if (!std::isfinite(v)) {
    o += "null";
    return;
  }
  char buf[40];
  for (int prec = 15; prec <= 17; ++prec) {
    std::snprintf(buf, sizeof(buf), "%.*g", prec, v);
    if (std::strtod(buf, nullptr) == v) break;
  }
  o += buf;
  if (!std::strpbrk(buf, ".eEn")) o += ".0";
}

void put_int(std::string& o, long long v) {
  char buf[32];
  std::snprintf(buf, sizeof(buf), "%lld", v);
  o += buf;
}

bool write_all(FILE* f, const std::string& s) {
  return std::fwrite(s.data(), 1, s.size(), f) == s.size();
}

}  // namespace

struct eqf_json {
  FILE* f = nullptr;
  long long frames = 0;
  long long time_since_epoch = 0;
  int node_id = 0, sim_number = 0;
};

extern "C" int eqf_json_open(const char* path, int64_t time_since_epoch, int32_t node_id,
                             int32_t sim_number, eqf_json** out) {
  if (!path || !out) return EQF_ERR_INVALID;
  FILE* f = std::fopen(path, "wb");
  if (!f) return EQF_ERR_INVALID;
  auto* j = new eqf_json;
  j->f = f;
  j->time_since_epoch = time_since_epoch;
  j->node_id = node_id;
  j->sim_number = sim_number;
  // keys in sorted order: cellDataFormat, frames, then the rest at close
  const std::string head =
      "{\"cellDataFormat\":[[\"id\",\"strainType\"],[\"x\",\"y\",\"angle\",\"length\","
      "\"spring\",\"vargs\"]],\"frames\":[";
  if (!write_all(f, head)) {
    std::fclose(f);
    delete j;
    return EQF_ERR_INVALID;
  }
  *out = j;
  return EQF_OK;
}

extern "C" int eqf_json_frame_host(eqf_json* j, int32_t n_layers, int64_t n_nodes,
                                   const double* fields, double sim_time, int64_t n_div,
                                   const double* divisions, int64_t n_cells, const int64_t* ids,
                                   int32_t n_data, const double* data) {
  if (!j || !j->f || n_layers < 0 || n_nodes < 0 || n_div < 0 || n_cells < 0 || n_data < 0)
    return EQF_ERR_INVALID;
  if ((n_layers > 0 && n_nodes > 0 && !fields) || (n_div > 0 && !divisions) ||
      (n_cells > 0 && (!ids || (n_data > 0 && !data))))
    return EQF_ERR_INVALID;
  std::string o;
  o.reserve(64 + (size_t)n_cells * (40 + 24 * n_data) + (size_t)n_layers * n_nodes * 24);
  if (j->frames > 0) o += ',';
  o += "{\"cells\":[";
  for (int64_t c = 0; c < n_cells; ++c) {
    if (c) o += ',';
    o += "[[";
    put_int(o, ids[2 * c]);
    o += ',';
    put_int(o, ids[2 * c + 1]);
    o += "],[";
    for (int32_t k = 0; k < n_data; ++k) {
      if (k) o += ',';
      put_double(o, data[(size_t)c * n_data + k]);
    }
    o += "]]";
  }
  o += "],\"divisions\":[";
  for (int64_t d = 0; d < n_div; ++d) {
    const double* e = divisions + 5 * d;  // time, parent id, its length, daughter id, its length
    if (d) o += ',';
    o += '[';
    put_double(o, e[0]);
    o += ',';
    put_int(o, (long long)std::llround(e[1]));
    o += ',';
    put_double(o, e[2]);
    o += ',';
    put_int(o, (long long)std::llround(e[3]));
    o += ',';
    put_double(o, e[4]);
    o += ']';
  }
  o += "],\"externalHSL\":[";
  for (int32_t l = 0; l < n_layers; ++l) {
    if (l) o += ',';
    o += '[';
    for (int64_t k = 0; k < n_nodes; ++k) {
      if (k) o += ',';
      put_double(o, fields[(size_t)l * n_nodes + k]);
    }
    o += ']';
  }
  o += "],\"simTime\":";
  put_double(o, sim_time);
  o += '}';
  if (!write_all(j->f, o)) return EQF_ERR_INVALID;
  ++j->frames;
  return EQF_OK;
}

extern "C" int eqf_json_frame(eqf_json* j, eqf_batch* b, int32_t n_layers, const int32_t* layers,
                              double sim_time, int64_t n_div, const double* divisions,
                              int64_t n_cells, const int64_t* ids, int32_t n_data,
                              const double* data) {
  if (!j || !b || n_layers < 0 || (n_layers > 0 && !layers)) return EQF_ERR_INVALID;
  int64_t nn = 0;
  std::vector<double> fields;
  for (int32_t l = 0; l < n_layers; ++l) {
    int64_t n = 0;
    int rc = eqf_num_nodes(b, layers[l], &n);
    if (rc != EQF_OK) return rc;
    if (l == 0) {
      nn = n;
      fields.resize((size_t)n_layers * nn);
    } else if (n != nn) {
      return EQF_ERR_INVALID;  // the layers of one recording share the mesh
    }
    rc = eqf_read_nodal(b, layers[l], fields.data() + (size_t)l * nn);
    if (rc != EQF_OK) return rc;
  }
  return eqf_json_frame_host(j, n_layers, nn, fields.data(), sim_time, n_div, divisions,
                             n_cells, ids, n_data, data);
}

extern "C" int eqf_json_close(eqf_json* j, const char* parameters_json) {
  if (!j) return EQF_ERR_INVALID;
  std::string o = "],\"jsonSimVersion\":\"v00_02\",\"nodeID\":";
  put_int(o, j->node_id);
  o += ",\"parameters\":";
  o += parameters_json ? parameters_json : "{}";
  o += ",\"simNumber\":";
  put_int(o, j->sim_number);
  o += ",\"timeSinceEpoch\":";
  put_int(o, j->time_since_epoch);
  o += "}\n";
  const bool ok = write_all(j->f, o);
  const bool closed = std::fclose(j->f) == 0;
  delete j;
  return ok && closed ? EQF_OK : EQF_ERR_INVALID;
}

// ---------------------------------------------------------------------------
struct eqf_vtk {
  std::string pvd, dir, stem;
  std::vector<std::pair<double, std::string>> steps;  // (time, file name)
};

extern "C" int eqf_vtk_open(const char* pvd_path, eqf_vtk** out) {
  if (!pvd_path || !out) return EQF_ERR_INVALID;
  std::string p(pvd_path);
  if (p.size() < 5 || p.compare(p.size() - 4, 4, ".pvd") != 0) return EQF_ERR_INVALID;
  auto* v = new eqf_vtk;
  v->pvd = p;
  const size_t slash = p.find_last_of('/');
  v->dir = slash == std::string::npos ? "" : p.substr(0, slash + 1);
  v->stem = p.substr(v->dir.size(), p.size() - v->dir.size() - 4);
  *out = v;
  return EQF_OK;
}

static int vtk_write_collection(const eqf_vtk* v) {
  std::string o =
      "<?xml version=\"1.0\"?>\n<VTKFile type=\"Collection\" version=\"0.1\">\n  <Collection>\n";
  for (const auto& s : v->steps) {
    o += "    <DataSet timestep=\"";
    put_double(o, s.first);
    o += "\" part=\"0\" file=\"" + s.second + "\" />\n";
  }
  o += "  </Collection>\n</VTKFile>\n";
  FILE* f = std::fopen(v->pvd.c_str(), "wb");
  if (!f) return EQF_ERR_INVALID;
  const bool ok = write_all(f, o);
  return std::fclose(f) == 0 && ok ? EQF_OK : EQF_ERR_INVALID;
}

extern "C" int eqf_vtk_write_host(eqf_vtk* v, double width, double height, int32_t nx, int32_t ny,
                                  const double* field, double time) {
  if (!v || !field || nx < 1 || ny < 0 || !(width > 0) || (ny > 0 && !(height > 0)))
    return EQF_ERR_INVALID;
  const long long np = (long long)(nx + 1) * (ny + 1);
  const long long nc = ny > 0 ? 2ll * nx * ny : nx;
  std::string o;
  o.reserve((size_t)np * 64 + (size_t)nc * 24 + 1024);
  o += "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\">\n"
       "  <UnstructuredGrid>\n    <Piece NumberOfPoints=\"";
  put_int(o, np);
  o += "\" NumberOfCells=\"";
  put_int(o, nc);
  o += "\">\n      <PointData Scalars=\"u\">\n"
       "        <DataArray type=\"Float64\" Name=\"u\" format=\"ascii\">";
  for (long long k = 0; k < np; ++k) {
    o += ' ';
    put_double(o, field[k]);
  }
  o += "</DataArray>\n      </PointData>\n      <Points>\n"
       "        <DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">";
  for (int i = 0; i <= ny; ++i)
    for (int j = 0; j <= nx; ++j) {  // vertex (i, j) at (j W / nx, i H / ny)
      o += ' ';
      put_double(o, j * (width / nx));
      o += ' ';
      put_double(o, ny > 0 ? i * (height / ny) : 0.0);
      o += " 0";
    }
  o += "</DataArray>\n      </Points>\n      <Cells>\n"
       "        <DataArray type=\"UInt32\" Name=\"connectivity\" format=\"ascii\">";
  if (ny > 0) {
    // each square (i, j) cut along (i, j)-(i+1, j+1): (v0, v1, v3) and (v0, v2, v3)
    for (int i = 0; i < ny; ++i)
      for (int j = 0; j < nx; ++j) {
        const long long v0 = j + (long long)i * (nx + 1), v1 = v0 + 1, v2 = v0 + nx + 1,
                        v3 = v2 + 1;
        const long long t[6] = {v0, v1, v3, v0, v2, v3};
        for (long long q : t) {
          o += ' ';
          put_int(o, q);
        }
      }
  } else {
    for (int j = 0; j < nx; ++j) {
      o += ' ';
      put_int(o, j);
      o += ' ';
      put_int(o, j + 1);
    }
  }
  o += "</DataArray>\n        <DataArray type=\"UInt32\" Name=\"offsets\" format=\"ascii\">";
  const int per = ny > 0 ? 3 : 2;
  for (long long c = 1; c <= nc; ++c) {
    o += ' ';
    put_int(o, c * per);
  }
  o += "</DataArray>\n        <DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">";
  for (long long c = 0; c < nc; ++c) o += ny > 0 ? " 5" : " 3";  // VTK_TRIANGLE / VTK_LINE
  o += "</DataArray>\n      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n";
  char num[16];
  std::snprintf(num, sizeof(num), "%06d", (int)v->steps.size());
  const std::string name = v->stem + num + ".vtu";
  FILE* f = std::fopen((v->dir + name).c_str(), "wb");
  if (!f) return EQF_ERR_INVALID;
  const bool ok = write_all(f, o);
  if (std::fclose(f) != 0 || !ok) return EQF_ERR_INVALID;
  v->steps.emplace_back(time, name);
  return vtk_write_collection(v);
}

extern "C" int eqf_vtk_write(eqf_vtk* v, eqf_batch* b, int32_t trap, double time) {
  if (!v || !b) return EQF_ERR_INVALID;
  eqf_trap_params p;
  int rc = eqf_trap_info(b, trap, &p);
  if (rc != EQF_OK) return rc;
  std::vector<double> u((size_t)(p.nx + 1) * (p.ny + 1));
  rc = eqf_read_nodal(b, trap, u.data());
  if (rc != EQF_OK) return rc;
  return eqf_vtk_write_host(v, p.width, p.height, p.nx, p.ny, u.data(), time);
}

extern "C" int eqf_vtk_write_channel(eqf_vtk* v, eqf_batch* b, int32_t trap, int32_t side,
                                     double time) {
  if (!v || !b || (side != EQF_SIDE_BOTTOM && side != EQF_SIDE_TOP)) return EQF_ERR_INVALID;
  eqf_trap_params p;
  int rc = eqf_trap_info(b, trap, &p);
  if (rc != EQF_OK) return rc;
  std::vector<double> c((size_t)p.nx + 1);
  rc = eqf_read_channels(b, trap, side == EQF_SIDE_BOTTOM ? c.data() : nullptr,
                         side == EQF_SIDE_TOP ? c.data() : nullptr);
  if (rc != EQF_OK) return rc;
  return eqf_vtk_write_host(v, p.width, 0.0, p.nx, 0, c.data(), time);
}

extern "C" int eqf_vtk_close(eqf_vtk* v) {
  if (!v) return EQF_ERR_INVALID;
  delete v;
  return EQF_OK;
}
