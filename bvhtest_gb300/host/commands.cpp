// The BVHTest commands over libbvhgb's C ABI. Each class cites the reference command it replaces;
// option names and defaults are the reference's, new keys are additive.
#include "commands.hpp"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <sstream>
#include <thread>

namespace fs = std::filesystem;

namespace bvhgb::host {

namespace {

std::string *g_log = nullptr;
bool g_verbose = true;

void logf(const char *level, const std::string &msg) {
  std::string line = std::string("[") + level + "] " + msg + "\n";
  if (g_log) *g_log += line;
  if (g_verbose || std::strcmp(level, "info") != 0) std::fputs(line.c_str(), stderr);
}
void info(const std::string &m) { logf("info", m); }
void warn(const std::string &m) { logf("warning", m); }
void error(const std::string &m) { logf("error", m); }

std::string cuda_detail() { return bvhgb_last_error(); }

bool read_file(const fs::path &p, std::string &out) {
  std::ifstream f(p, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

void vec3_from(const Json &j, float *v) {
  v[0] = j.value("x", v[0]);
  v[1] = j.value("y", v[1]);
  v[2] = j.value("z", v[2]);
}
Json vec3_to(const float *v) {
  Json o = Json::object();
  o["x"] = v[0];
  o["y"] = v[1];
  o["z"] = v[2];
  return o;
}

// Directory the IO commands work in: basePath/input, or its parent when input is a file.
bool io_dir(const State &s, fs::path &out) {
  fs::path p = fs::path(s.basePath) / s.input;
  if (fs::is_directory(p)) {
    out = p;
    return true;
  }
  if (fs::is_regular_file(p) && fs::is_directory(p.parent_path())) {
    out = p.parent_path();
    return true;
  }
  return false;
}

uint32_t adler32(const uint8_t *d, size_t n) {  // RFC 1950
  uint32_t a = 1, b = 0;
  for (size_t i = 0; i < n; ++i) {
    a = (a + d[i]) % 65521u;
    b = (b + a) % 65521u;
  }
  return (b << 16) | a;
}

// ---- IO -------------------------------------------------------------------------------------

// load (lib/io/Load.cpp:122-187): data.json {version 3, bin, mesh{vert, normals, faces}} + raw
// vec3 vert[], vec3 norm[], uint3 faces[].
class Load : public Command {
 public:
  std::string name() const override { return "load"; }
  std::string desc() const override { return "Load a mesh from the binary (data.json + bin) format"; }
  uint64_t type() const override { return IMPORT; }
  uint64_t required() const override { return 0; }

 protected:
  ErrorCode runImpl(State &s) override {
    fs::path p = fs::absolute(fs::path(s.basePath) / s.input);
    if (fs::is_directory(p)) p /= "data.json";
    std::string text;
    if (!read_file(p, text)) {
      error("File " + p.string() + " does not exist");
      return ErrorCode::IO_ERROR;
    }
    Json cfg;
    try {
      cfg = Json::parse(text);
      uint32_t vers = (uint32_t)cfg.at("version").as_number();
      if (vers != 3) {
        error("File format version is " + std::to_string(vers) + " but 3 is required");
        return ErrorCode::PARSE_ERROR;
      }
      fs::path bin = p.parent_path() / cfg.at("bin").as_string();
      size_t nv = (size_t)cfg.at("mesh").at("vert").as_number();
      size_t nn = (size_t)cfg.at("mesh").at("normals").as_number();
      size_t nf = (size_t)cfg.at("mesh").at("faces").as_number();
      std::ifstream f(bin, std::ios::binary);
      if (!f) {
        error("File " + bin.string() + " does not exist");
        return ErrorCode::IO_ERROR;
      }
      s.vert.resize(3 * nv);
      s.norm.resize(3 * nn);
      s.faces.resize(3 * nf);
      f.read(reinterpret_cast<char *>(s.vert.data()), (std::streamsize)(12 * nv));
      f.read(reinterpret_cast<char *>(s.norm.data()), (std::streamsize)(12 * nn));
      f.read(reinterpret_cast<char *>(s.faces.data()), (std::streamsize)(12 * nf));
      if (!f) {
        error("Binary file " + bin.string() + " is too short");
        return ErrorCode::IO_ERROR;
      }
    } catch (const JsonError &e) {
      error(e.what());
      return ErrorCode::PARSE_ERROR;
    }
    return ErrorCode::OK;
  }
};

// Seeded synthetic scenes (an addition; the reference's mesh files are not distributed): a soup of
// independent triangles, centroids uniform in [0,1]^3 (or a Gaussian mixture), vertex offsets
// N(0, sigma^2). SplitMix64 + Box-Muller; adds a default camera when none is loaded.
class Generate : public Command {
  std::string vScene = "uniform";
  uint32_t vTriangles = 65536, vSeed = 1, vClusters = 64;
  float vSigma = 0.004f;

 public:
  std::string name() const override { return "generate"; }
  std::string desc() const override { return "Generate a seeded synthetic triangle soup"; }
  uint64_t type() const override { return IMPORT; }
  uint64_t required() const override { return 0; }
  void fromJSON(const Json &j) override {
    vScene = j.value("scene", vScene);
    vTriangles = j.value("triangles", vTriangles);
    vSeed = j.value("seed", vSeed);
    vClusters = j.value("clusters", vClusters);
    vSigma = j.value("sigma", vSigma);
  }
  Json toJSON() const override {
    Json o = Json::object();
    o["scene"] = vScene;
    o["triangles"] = vTriangles;
    o["seed"] = vSeed;
    o["clusters"] = vClusters;
    o["sigma"] = vSigma;
    return o;
  }

 protected:
  ErrorCode runImpl(State &s) override {
    uint64_t st = 0x243F6A8885A308D3ull ^ vSeed;
    auto next = [&]() {
      uint64_t z = (st += 0x9E3779B97F4A7C15ull);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      return z ^ (z >> 31);
    };
    auto uni = [&]() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); };
    auto gauss = [&]() {
      double u1 = uni(), u2 = uni();
      if (u1 < 1e-300) u1 = 1e-300;
      return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    };
    const bool gmm = vScene == "gmm";
    std::vector<double> mean(3 * (gmm ? vClusters : 1)), sig(gmm ? vClusters : 1);
    if (gmm) {
      for (auto &m : mean) m = uni() * 10.0;
      for (auto &g : sig) g = std::exp(std::log(0.05) + uni() * (std::log(0.8) - std::log(0.05)));
    } else if (vScene != "uniform") {
      error("unknown scene '" + vScene + "' (uniform | gmm)");
      return ErrorCode::PARSE_ERROR;
    }
    s.vert.resize(9ull * vTriangles);
    s.faces.resize(3ull * vTriangles);
    s.norm.clear();
    const double vs = gmm ? 0.01 : vSigma;
    for (uint32_t t = 0; t < vTriangles; ++t) {
      double c[3];
      if (gmm) {
        uint32_t k = (uint32_t)(next() % vClusters);
        for (int a = 0; a < 3; ++a) c[a] = mean[3 * k + a] + gauss() * sig[k];
      } else {
        for (int a = 0; a < 3; ++a) c[a] = uni();
      }
      for (int v = 0; v < 3; ++v) {
        for (int a = 0; a < 3; ++a) s.vert[9ull * t + 3 * v + a] = (float)(c[a] + gauss() * vs);
        s.faces[3ull * t + v] = 3 * t + v;
      }
    }
    if (s.cameras.empty()) {
      CameraDesc c;
      const float p[3] = {0.5f, 0.5f, -1.5f}, l[3] = {0.5f, 0.5f, 0.0f};
      if (gmm) {
        const float gp[3] = {5.0f, 5.0f, -12.0f}, gl[3] = {5.0f, 5.0f, 5.0f};
        std::memcpy(c.pos, gp, 12);
        std::memcpy(c.lookAt, gl, 12);
      } else {
        std::memcpy(c.pos, p, 12);
        std::memcpy(c.lookAt, l, 12);
      }
      c.fov = 60.0f;
      c.width = c.height = 512;
      s.cameras.push_back(c);
    }
    return ErrorCode::OK;
  }
};

// camImport (lib/io/CameraImport.cpp:42-108): cameras.json {version 1, cameras[{type, cam}]}.
class CamImport : public Command {
  bool vAbortOnError = true;

 public:
  std::string name() const override { return "camImport"; }
  std::string desc() const override { return "Import cameras from cameras.json"; }
  uint64_t type() const override { return IMPORT; }
  uint64_t required() const override { return 0; }
  void fromJSON(const Json &j) override { vAbortOnError = j.value("abortOnError", vAbortOnError); }
  Json toJSON() const override {
    Json o = Json::object();
    o["abortOnError"] = vAbortOnError;
    return o;
  }

 protected:
  ErrorCode runImpl(State &s) override {
    const ErrorCode fail = vAbortOnError ? ErrorCode::IO_ERROR : ErrorCode::OK;
    fs::path dir;
    if (!io_dir(s, dir)) {
      error("Invalid base path " + (fs::path(s.basePath) / s.input).string());
      return fail;
    }
    std::string text;
    if (!read_file(dir / "cameras.json", text)) {
      error("Path '" + (dir / "cameras.json").string() + "' is not a regular file");
      return fail;
    }
    try {
      Json d = Json::parse(text);
      if ((uint32_t)d.at("version").as_number() != 1) {
        error("Incompatible camera file version");
        return fail;
      }
      for (const Json &c : d.at("cameras").as_array()) {
        if (c.at("type").as_string() != "PERSPECTIVE") {
          warn("Currently only PERSPECTIVE type cameras supported");
          continue;
        }
        CameraDesc cd;
        cd.fromJSON(c.at("cam"));
        s.cameras.push_back(cd);
      }
    } catch (const JsonError &e) {
      error(e.what());
      return fail;
    }
    return ErrorCode::OK;
  }
};

// BVHExport / BVHImport (lib/io/BVHExport.cpp:44-117, BVHImport.cpp:42-141): <name>_bvh.json
// {version 9, bin, BVHSize, treeHeight, rawChecksum (adler32)} + raw 48-byte nodes.
class BVHExport : public Command {
  std::string vName = "genericBVH";

 public:
  std::string name() const override { return "BVHExport"; }
  std::string desc() const override { return "Export a built BVH in binary format"; }
  uint64_t type() const override { return EXPORT; }
  uint64_t required() const override { return BVH_BUILD; }
  void fromJSON(const Json &j) override { vName = j.value("name", vName); }
  Json toJSON() const override {
    Json o = Json::object();
    o["name"] = vName;
    return o;
  }

 protected:
  ErrorCode runImpl(State &s) override {
    fs::path dir;
    if (!io_dir(s, dir)) return ErrorCode::IO_ERROR;
    const auto *raw = reinterpret_cast<const uint8_t *>(s.bvh.data());
    const size_t bytes = s.bvh.size() * sizeof(bvhgb_node);
    Json c = Json::object();
    c["version"] = 9;
    c["bin"] = vName + "_bvh.bin";
    c["BVHSize"] = (uint64_t)s.bvh.size();
    c["treeHeight"] = (uint32_t)s.maxLevel;
    c["rawChecksum"] = adler32(raw, bytes);
    std::ofstream jf(dir / (vName + "_bvh.json"), std::ios::trunc);
    std::ofstream bf(dir / (vName + "_bvh.bin"), std::ios::binary | std::ios::trunc);
    if (!jf || !bf) return ErrorCode::IO_ERROR;
    jf << c.dump(2);
    bf.write(reinterpret_cast<const char *>(raw), (std::streamsize)bytes);
    return (jf && bf) ? ErrorCode::OK : ErrorCode::IO_ERROR;
  }
};

class BVHImport : public Command {
  std::string vName = "genericBVH";

 public:
  std::string name() const override { return "BVHImport"; }
  std::string desc() const override { return "Import a BVH exported by BVHExport"; }
  uint64_t type() const override { return BVH_BUILD; }
  uint64_t required() const override { return IMPORT; }
  void fromJSON(const Json &j) override { vName = j.value("name", vName); }
  Json toJSON() const override {
    Json o = Json::object();
    o["name"] = vName;
    return o;
  }

 protected:
  ErrorCode runImpl(State &s) override {
    fs::path dir;
    if (!io_dir(s, dir)) return ErrorCode::IO_ERROR;
    std::string text;
    if (!read_file(dir / (vName + "_bvh.json"), text)) return ErrorCode::IO_ERROR;
    try {
      Json c = Json::parse(text);
      if ((uint32_t)c.at("version").as_number() != 9) return ErrorCode::PARSE_ERROR;
      const size_t n = (size_t)c.at("BVHSize").as_number();
      std::ifstream bf(dir / c.at("bin").as_string(), std::ios::binary);
      if (!bf) return ErrorCode::IO_ERROR;
      s.bvh.resize(n);
      bf.read(reinterpret_cast<char *>(s.bvh.data()), (std::streamsize)(n * sizeof(bvhgb_node)));
      if (!bf) return ErrorCode::IO_ERROR;
      if (adler32(reinterpret_cast<const uint8_t *>(s.bvh.data()), n * sizeof(bvhgb_node)) !=
          (uint32_t)c.at("rawChecksum").as_number()) {
        error("corrupt BVH binary");
        return ErrorCode::IO_ERROR;
      }
      s.maxLevel = (uint16_t)c.value("treeHeight", 0.0);
      s.root = 0;
    } catch (const JsonError &e) {
      error(e.what());
      return ErrorCode::PARSE_ERROR;
    }
    return ErrorCode::OK;
  }
};

// writeData (lib/io/WriteData.cpp:40-84): %d = basePath, %i = input, %n = config name.
class WriteData : public Command {
  std::string vOutFile = "%d/%i/rData_%n.json";

 public:
  std::string name() const override { return "writeData"; }
  std::string desc() const override { return "Write optimizer statistics as JSON"; }
  uint64_t type() const override { return EXPORT; }
  uint64_t required() const override { return 0; }
  void fromJSON(const Json &j) override { vOutFile = j.value("outFile", vOutFile); }
  Json toJSON() const override {
    Json o = Json::object();
    o["outFile"] = vOutFile;
    return o;
  }

 protected:
  static void subst(std::string &s, const std::string &from, const std::string &to) {
    for (size_t p = s.find(from); p != std::string::npos; p = s.find(from, p + to.size())) s.replace(p, from.size(), to);
  }
  ErrorCode runImpl(State &s) override {
    if (!fs::is_directory(s.basePath)) return ErrorCode::IO_ERROR;
    std::string f = vOutFile;
    subst(f, "%d", s.basePath);
    subst(f, "%i", s.input);
    subst(f, "%n", s.name);
    double total = 0.0;
    for (const auto &c : s.commands)
      if (c.type == BVH_OPT1 || c.type == BVH_OPT2) total = c.ms;
    Json steps = Json::array();
    for (const auto &o : s.optData.optStepps) {
      Json e = Json::object();
      e["step"] = o.step;
      e["sah"] = o.sah;
      e["duration"] = (int64_t)o.ms;
      steps.push_back(e);
    }
    Json d = Json::object();
    d["totalTime"] = (int64_t)total;
    d["optStepps"] = steps;
    d["numSkipped"] = s.optData.numSkipped;
    d["numTotal"] = s.optData.numTotal;
    d["numFaces"] = (uint64_t)(s.faces.size() / 3);
    d["numVert"] = (uint64_t)(s.vert.size() / 3);
    d["numBVHNodes"] = (uint64_t)s.bvh.size();
    std::ofstream out(f, std::ios::trunc);
    if (!out) return ErrorCode::IO_ERROR;
    out << d.dump(2);
    return out ? ErrorCode::OK : ErrorCode::IO_ERROR;
  }
};

// writeImg: the reference writes PNG through lodepng (absent); this writes binary PPM with the same
// colours (CUDATracer.cpp:133-146: grey diffuse on hits, (121,167,229) background).
class WriteImg : public Command {
 public:
  std::string name() const override { return "writeImg"; }
  std::string desc() const override { return "Write traced images (PPM)"; }
  uint64_t type() const override { return EXPORT; }
  uint64_t required() const override { return RAY_TRACE; }

 protected:
  ErrorCode runImpl(State &s) override {
    for (const auto &w : s.work) {
      std::ofstream f(fs::path(s.basePath) / (w.name + ".ppm"), std::ios::binary | std::ios::trunc);
      if (!f) return ErrorCode::IO_ERROR;
      f << "P6\n" << w.width << " " << w.height << "\n255\n";
      for (const auto &p : w.pixels) {
        const unsigned char c[3] = {p.hit ? p.diffuse : (unsigned char)121, p.hit ? p.diffuse : (unsigned char)167,
                                    p.hit ? p.diffuse : (unsigned char)229};
        f.write(reinterpret_cast<const char *>(c), 3);
      }
    }
    return ErrorCode::OK;
  }
};

// ---- CUDA transfer ----------------------------------------------------------------------------

// copyToGPU (lib/cuda/CopyToGPU.cpp:30-34).
class CopyToGPU : public Command {
 public:
  std::string name() const override { return "copyToGPU"; }
  std::string desc() const override { return "Copy mesh (and BVH) to the GPU"; }
  uint64_t type() const override { return CUDA_INIT; }
  uint64_t required() const override { return IMPORT; }

 protected:
  ErrorCode runImpl(State &s) override {
    int st = bvhgb_copy_bvh_to_gpu(s.bvh.data(), (uint32_t)s.bvh.size(), s.root, s.maxLevel, &s.cudaBVH);
    if (st) {
      error("copyBVHToGPU: " + cuda_detail());
      return ErrorCode::CUDA_ERROR;
    }
    st = bvhgb_copy_mesh_to_gpu(s.vert.data(), (uint32_t)(s.vert.size() / 3), s.norm.data(),
                                (uint32_t)(s.norm.size() / 3), s.faces.data(), (uint32_t)(s.faces.size() / 3),
                                &s.rawMesh);
    if (st) {
      error("copyMeshToGPU: " + cuda_detail());
      return ErrorCode::CUDA_ERROR;
    }
    return ErrorCode::OK;
  }
};

// copyToHost (lib/cuda/CopyToHost.cpp:30-36).
class CopyToHost : public Command {
  bool vFixLevels = true;

 public:
  std::string name() const override { return "copyToHost"; }
  std::string desc() const override { return "Copy the BVH (and mesh) back and release the GPU data"; }
  uint64_t type() const override { return CUDA_DONE; }
  uint64_t required() const override { return CUDA_INIT; }
  void fromJSON(const Json &j) override { vFixLevels = j.value("fixLevels", vFixLevels); }
  Json toJSON() const override {
    Json o = Json::object();
    o["fixLevels"] = vFixLevels;
    return o;
  }

 protected:
  ErrorCode runImpl(State &s) override {
    if (s.cudaBVH.nodes) {
      s.bvh.resize(s.cudaBVH.numNodes);
      uint32_t root = 0;
      uint16_t ml = 0;
      if (bvhgb_copy_bvh_to_host(&s.cudaBVH, s.bvh.data(), (uint32_t)s.bvh.size(), &root, &ml)) return ErrorCode::CUDA_ERROR;
      s.root = root;
      s.maxLevel = ml;
    }
    if (s.rawMesh.vert) {
      if (bvhgb_copy_mesh_to_host(&s.rawMesh, s.vert.data(), s.norm.empty() ? nullptr : s.norm.data(), s.faces.data()))
        return ErrorCode::CUDA_ERROR;
    }
    if (vFixLevels && !s.bvh.empty()) {
      uint16_t ml = 0;
      if (bvhgb_fix_levels_host(s.bvh.data(), (uint32_t)s.bvh.size(), s.root, &ml)) return ErrorCode::BVH_ERROR;
      s.maxLevel = ml;
    }
    return ErrorCode::OK;
  }
};

// ---- builders ---------------------------------------------------------------------------------

// LBVH (lib/builder/LBVH.cpp:25-55): costInner / costLeaf are kept for config compatibility
// (unused by the LBVH build, as in the reference); mortonBits / topology are additions.
class LBVH : public Command {
  float vCostInner = 1.2f, vCostLeaf = 1.0f;
  uint32_t vMortonBits = 30;
  std::string vTopology = "refCompat";
  bvhgb_lbvh_workspace *vWs = nullptr;

 public:
  std::string name() const override { return "LBVH"; }
  std::string desc() const override { return "LBVH CUDA builder"; }
  uint64_t type() const override { return BVH_BUILD; }
  uint64_t required() const override { return IMPORT | CUDA_INIT; }
  void fromJSON(const Json &j) override {
    vCostInner = j.value("costInner", vCostInner);
    vCostLeaf = j.value("costLeaf", vCostLeaf);
    vMortonBits = j.value("mortonBits", vMortonBits);
    vTopology = j.value("topology", vTopology);
  }
  Json toJSON() const override {
    Json o = Json::object();
    o["costInner"] = vCostInner;
    o["costLeaf"] = vCostLeaf;
    o["mortonBits"] = vMortonBits;
    o["topology"] = vTopology;
    return o;
  }

 protected:
  ErrorCode setup(State &s) override {
    bvhgb_lbvh_config cfg{vMortonBits, vTopology == "karras" ? (uint32_t)BVHGB_TOPO_KARRAS : (uint32_t)BVHGB_TOPO_REFCOMPAT};
    if (vTopology != "karras" && vTopology != "refCompat") {
      error("topology must be refCompat or karras");
      return ErrorCode::PARSE_ERROR;
    }
    int st = bvhgb_lbvh_create(s.rawMesh.numFaces, &cfg, &vWs);
    if (st) return from_status(st);
    bvhgb_free_bvh(&s.cudaBVH);  // an imported BVH on the GPU is replaced
    st = bvhgb_allocate_bvh(&s.cudaBVH, s.rawMesh.numFaces);
    if (st) {
      bvhgb_lbvh_destroy(vWs);
      vWs = nullptr;
      return from_status(st);
    }
    return ErrorCode::OK;
  }
  ErrorCode runImpl(State &s) override {
    int st = bvhgb_lbvh_build(vWs, reinterpret_cast<const float *>(s.rawMesh.vert),
                              reinterpret_cast<const uint32_t *>(s.rawMesh.faces), s.rawMesh.numFaces, s.cudaBVH.nodes,
                              nullptr);
    if (st == BVHGB_OK) st = bvhgb_device_sync();
    uint32_t flags = 0;
    if (st == BVHGB_OK && bvhgb_lbvh_read_errors(vWs, &flags, nullptr) == BVHGB_OK && flags) st = BVHGB_DEVICE_TIMEOUT;
    s.root = 0;
    return from_status(st);
  }
  void teardown(State &) override {
    bvhgb_lbvh_destroy(vWs);
    vWs = nullptr;
  }
};

// bittner13GPU (lib/builder/Bittner13GPU.cpp:46-133, OptimizerBase.cpp:28-57).
class Bittner13GPU : public Command {
  bool vCalcSAH = false, vDoSync = false;
  uint32_t vMaxNumStepps = 500, vNumChunks = 32, vBlockSize = 128;
  float vBatchPercent = 1.0f;
  bool vSort = true, vOffsetAccess = false, vAltFindNode = false, vAltFixTree = false, vAltSort = false,
       vLocalPatchCPY = false;
  std::string vSearch = "batched";
  std::string vScorer;  // learned scorer weights (5825 little-endian float32); empty = inefficiency
  uint32_t vPlainEvery = 2;  // with a scorer: every k-th iteration selects by the inefficiency
  bvhgb_bn13_workspace *vWs = nullptr;
  bvhgb_mlp *vMlp = nullptr;

 public:
  std::string name() const override { return "bittner13GPU"; }
  std::string desc() const override { return "CUDA: parallel BVH optimizer based on Bittner et al. 2013"; }
  uint64_t type() const override { return BVH_OPT1; }
  uint64_t required() const override { return BVH_BUILD | CUDA_INIT; }
  void fromJSON(const Json &j) override {
    vCalcSAH = j.value("base_calcSAH", vCalcSAH);
    vDoSync = j.value("base_doSync", vDoSync);
    vMaxNumStepps = j.value("maxNumStepps", vMaxNumStepps);
    vNumChunks = j.value("numChunks", vNumChunks);
    vBlockSize = j.value("CUDABlockSize", vBlockSize);
    vBatchPercent = j.value("batchPercent", vBatchPercent);
    vSort = j.value("sort", vSort);
    vOffsetAccess = j.value("offsetAccess", vOffsetAccess);
    vAltFindNode = j.value("altFindNode", vAltFindNode);
    vAltFixTree = j.value("altFixTree", vAltFixTree);
    vAltSort = j.value("altSort", vAltSort);
    vLocalPatchCPY = j.value("localPatchCPY", vLocalPatchCPY);
    vSearch = j.value("searchMode", vSearch);
    vScorer = j.value("learnedScorer", vScorer);
    vPlainEvery = j.value("learnedPlainEvery", vPlainEvery);
    if (vBatchPercent <= 0.01f) vBatchPercent = 0.01f;
    if (vBatchPercent >= 75.0f) vBatchPercent = 75.0f;
  }
  Json toJSON() const override {
    Json o = Json::object();
    o["base_calcSAH"] = vCalcSAH;
    o["base_doSync"] = vDoSync;
    o["maxNumStepps"] = vMaxNumStepps;
    o["numChunks"] = vNumChunks;
    o["CUDABlockSize"] = vBlockSize;
    o["batchPercent"] = vBatchPercent;
    o["sort"] = vSort;
    o["offsetAccess"] = vOffsetAccess;
    o["altFindNode"] = vAltFindNode;
    o["altFixTree"] = vAltFixTree;
    o["altSort"] = vAltSort;
    o["localPatchCPY"] = vLocalPatchCPY;
    o["searchMode"] = vSearch;
    o["learnedScorer"] = vScorer;
    o["learnedPlainEvery"] = vPlainEvery;
    return o;
  }

 protected:
  float sah(State &s) {
    double v = 0.0;
    bvhgb_calc_sah(s.cudaBVH.nodes, s.cudaBVH.numNodes, s.root, &v, nullptr);
    return (float)v;
  }
  ErrorCode setup(State &s) override {
    if (!vSort) {
      error("sort = false is not supported (the reference reports the same: Bittner13CUDA.cu:719)");
      return ErrorCode::GENERIC_ERROR;
    }
    // altFindNode selects the reference's approximate 16-slot search (findNode2); otherwise
    // searchMode picks the batched (default) or the heap (findNode1) search.
    const uint32_t mode = vAltFindNode || vSearch == "alt" ? (uint32_t)BVHGB_SEARCH_ALT
                          : vSearch == "heap"              ? (uint32_t)BVHGB_SEARCH_HEAP
                                                           : (uint32_t)BVHGB_SEARCH_BATCHED;
    bvhgb_bn13_config cfg{vNumChunks, vBlockSize, vBatchPercent, vOffsetAccess ? 1u : 0u, 4096u, 0u, mode};
    ErrorCode e = from_status(bvhgb_bn13_create(s.cudaBVH.nodes, s.cudaBVH.numNodes, s.root, &cfg, &vWs, nullptr));
    if (e != ErrorCode::OK || vScorer.empty()) return e;
    // learned selection: weights relative to the base path unless absolute
    fs::path wp = fs::path(vScorer);
    if (wp.is_relative()) wp = fs::path(s.basePath) / wp;
    std::ifstream in(wp, std::ios::binary);
    std::vector<float> w(BVHGB_MLP_PARAMS);
    if (!in.read(reinterpret_cast<char *>(w.data()), (std::streamsize)(w.size() * sizeof(float)))) {
      error("learnedScorer: cannot read " + std::to_string(BVHGB_MLP_PARAMS) + " floats from " + wp.string());
      return ErrorCode::IO_ERROR;
    }
    int st = bvhgb_mlp_create(0, &vMlp);
    if (!st) st = bvhgb_mlp_set_params(vMlp, w.data());
    if (!st) st = bvhgb_bn13_set_scorer(vWs, vMlp, vPlainEvery);
    if (!st) info("learned selection with " + wp.string());
    return from_status(st);
  }
  ErrorCode runImpl(State &s) override {
    using clk = std::chrono::steady_clock;
    s.optData.numSkipped = s.optData.numTotal = 0;
    s.optData.optStepps.push_back({0u, vCalcSAH ? sah(s) : 0.0f, 0.0});
    if (vDoSync) bvhgb_device_sync();
    for (uint32_t i = 0; i < vMaxNumStepps; ++i) {
      s.optData.optStepps.push_back({(uint32_t)s.optData.optStepps.size(), 0.0f, 0.0});
      if (vDoSync) bvhgb_device_sync();
      auto t0 = clk::now();
      int st = bvhgb_bn13_run(vWs, s.cudaBVH.nodes, 1, nullptr);
      if (st) return from_status(st);
      if (vDoSync) bvhgb_device_sync();
      s.optData.optStepps.back().ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
      if (vCalcSAH) s.optData.optStepps.back().sah = sah(s);
    }
    return from_status(bvhgb_device_sync());
  }
  void teardown(State &s) override {
    bvhgb_bn13_stats st{};
    bvhgb_bn13_get_stats(vWs, &st, nullptr);
    s.optData.numSkipped = st.skippedConflict;
    s.optData.numTotal = (uint64_t)bvhgb_bn13_batch_size(vWs) * vMaxNumStepps;
    info("Skipped " + std::to_string(st.skippedConflict) + " of " + std::to_string(s.optData.numTotal));
    bvhgb_bn13_destroy(vWs);
    vWs = nullptr;
    bvhgb_mlp_destroy(vMlp);
    vMlp = nullptr;
  }
};

// ---- tracer -----------------------------------------------------------------------------------

// CUDATracer (lib/tracer/CUDATracer.cpp:31-150, TracerBase.cpp:39-50).
class CUDATracer : public Command {
  float vLight[3] = {2.0f, 2.0f, 2.0f};
  bool vRayBundles = false, vFaceCulling = false;

 public:
  std::string name() const override { return "CUDATracer"; }
  std::string desc() const override { return "CUDA closest-hit ray tracer"; }
  uint64_t type() const override { return RAY_TRACE; }
  uint64_t required() const override { return BVH_BUILD | CUDA_INIT; }
  void fromJSON(const Json &j) override {
    if (j.contains("lightLocation")) vec3_from(j.at("lightLocation"), vLight);
    vRayBundles = j.value("rayBundles", vRayBundles);
    vFaceCulling = j.value("faceCulling", vFaceCulling);
  }
  Json toJSON() const override {
    Json o = Json::object();
    o["lightLocation"] = vec3_to(vLight);
    o["rayBundles"] = vRayBundles;
    o["faceCulling"] = vFaceCulling;
    return o;
  }

 protected:
  ErrorCode setup(State &s) override {
    if (s.cameras.empty()) return ErrorCode::WARNING;  // CUDATracer.cpp:76-77
    return ErrorCode::OK;
  }
  ErrorCode runImpl(State &s) override;
};

// validate (lib/misc/Validate.cpp:42-277) on the host BVH.
class Validate : public Command {
 public:
  std::string name() const override { return "validate"; }
  std::string desc() const override { return "Validate the BVH (tree, boxes, surface areas, triangles)"; }
  uint64_t type() const override { return SUMMARY; }
  uint64_t required() const override { return BVH_BUILD; }

 protected:
  ErrorCode runImpl(State &s) override;
};

// status (lib/base/StatusDump.cpp:31-56).
class Status : public Command {
 public:
  std::string name() const override { return "status"; }
  std::string desc() const override { return "Print a summary of the state"; }
  uint64_t type() const override { return SUMMARY; }
  uint64_t required() const override { return 0; }

 protected:
  ErrorCode runImpl(State &s) override {
    double sumAll = 0.0;
    for (size_t i = 0; i < s.bvh.size(); ++i)
      if (i != s.root) sumAll += s.bvh[i].surfaceArea;
    const double sah = s.bvh.empty() ? -1.0 : sumAll / s.bvh[s.root].surfaceArea;
    std::ostringstream o;
    o << "Status:\n  -- BVH:\n    - Nodes:       " << s.bvh.size() << "\n    - Tree height: " << s.maxLevel
      << "\n    - SAH:         " << sah << "\n  -- Mesh info:\n    - Vertices: " << s.vert.size() / 3
      << "\n    - Faces:    " << s.faces.size() / 3 << "\n  -- Num Images: " << s.work.size() << "\n";
    for (const auto &w : s.work) o << "    - Image " << w.name << " -- Time: " << w.ns / 1e6 << " ms\n";
    o << "  -- Command times:\n";
    for (const auto &c : s.commands) o << "    - " << c.name << " -- " << c.ms << " ms\n";
    info(o.str());
    return ErrorCode::OK;
  }
};

// sleep (lib/misc/Sleep.cpp).
class Sleep : public Command {
  uint32_t vMs = 1000;

 public:
  std::string name() const override { return "sleep"; }
  std::string desc() const override { return "Sleep for a number of milliseconds"; }
  uint64_t type() const override { return SUMMARY; }
  uint64_t required() const override { return 0; }
  void fromJSON(const Json &j) override { vMs = j.value("ms", vMs); }
  Json toJSON() const override {
    Json o = Json::object();
    o["ms"] = vMs;
    return o;
  }

 protected:
  ErrorCode runImpl(State &) override {
    std::this_thread::sleep_for(std::chrono::milliseconds(vMs));
    return ErrorCode::OK;
  }
};

}  // namespace

// ---- shared pieces ------------------------------------------------------------------------------

const char *to_string(ErrorCode e) {
  switch (e) {
    case ErrorCode::OK: return "OK";
    case ErrorCode::WARNING: return "WARNING";
    case ErrorCode::IO_ERROR: return "IO_ERROR";
    case ErrorCode::PARSE_ERROR: return "PARSE_ERROR";
    case ErrorCode::BVH_ERROR: return "BVH_ERROR";
    case ErrorCode::GL_ERROR: return "GL_ERROR";
    case ErrorCode::CUDA_ERROR: return "CUDA_ERROR";
    default: return "GENERIC_ERROR";
  }
}

ErrorCode from_status(int st) {
  if (st >= 0 && st <= 7) return static_cast<ErrorCode>(st);
  if (st == BVHGB_INVALID_ARGUMENT || st == BVHGB_TOO_LARGE) return ErrorCode::GENERIC_ERROR;
  return ErrorCode::CUDA_ERROR;
}

void CameraDesc::fromJSON(const Json &j) {
  Json cam = j.value("camera", Json::object()), res = j.value("resolution", Json::object());
  vec3_from(cam.value("pos", Json::object()), pos);
  vec3_from(cam.value("lookAt", Json::object()), lookAt);
  vec3_from(cam.value("up", Json::object()), up);
  fov = cam.value("fov", fov);
  width = res.value("width", width);
  height = res.value("height", height);
}

Json CameraDesc::toJSON() const {
  Json cam = Json::object();
  cam["pos"] = vec3_to(pos);
  cam["lookAt"] = vec3_to(lookAt);
  cam["up"] = vec3_to(up);
  cam["fov"] = fov;
  Json res = Json::object();
  res["width"] = width;
  res["height"] = height;
  Json o = Json::object();
  o["camera"] = cam;
  o["resolution"] = res;
  return o;
}

State::~State() {
  bvhgb_free_bvh(&cudaBVH);
  if (rawMesh.vert || rawMesh.faces) bvhgb_free_mesh(&rawMesh);
}

ErrorCode Command::run(State &s) {
  info("Running:  command " + name() + " -- " + desc());
  if ((s.commandsRun & required()) != required())
    error("Command " + name() + " has unmet requirements");  // logged only, as the reference does
  ErrorCode r = setup(s);
  if (r != ErrorCode::OK) {
    error("Setup function of command " + name() + " returned " + to_string(r));
    return r;
  }
  auto t0 = std::chrono::steady_clock::now();
  r = runImpl(s);
  auto t1 = std::chrono::steady_clock::now();
  teardown(s);
  if (r == ErrorCode::WARNING) warn("Command " + name() + " returned a warning");
  if (r != ErrorCode::OK && r != ErrorCode::WARNING) {
    error("Command " + name() + " returned " + to_string(r) + (r == ErrorCode::CUDA_ERROR ? " (" + cuda_detail() + ")" : ""));
    return r;
  }
  s.commandsRun |= type();
  s.commands.push_back({name(), type(), std::chrono::duration<double, std::milli>(t1 - t0).count()});
  return ErrorCode::OK;
}

ErrorCode CUDATracer::runImpl(State &s) {
  for (size_t i = 0; i < s.cameras.size(); ++i) {
    const CameraDesc &c = s.cameras[i];
    bvhgb_camera cam{};
    std::memcpy(cam.pos, c.pos, 12);
    std::memcpy(cam.lookAt, c.lookAt, 12);
    std::memcpy(cam.up, c.up, 12);
    cam.fov = c.fov;
    cam.width = c.width;
    cam.height = c.height;
    bvhgb_trace_config tc{{vLight[0], vLight[1], vLight[2]}, vFaceCulling ? 1u : 0u, 0.0f, INFINITY,
                          vRayBundles ? 1u : 0u};
    const size_t npx = (size_t)c.width * c.height;
    bvhgb_pixel *img = nullptr;
    bvhgb_hit *hits = nullptr;
    if (cudaMalloc(&img, npx * sizeof(bvhgb_pixel)) != cudaSuccess ||
        cudaMalloc(&hits, npx * sizeof(bvhgb_hit)) != cudaSuccess) {
      cudaFree(img);
      return ErrorCode::CUDA_ERROR;
    }
    State::Work w;
    w.name = s.name + "_CUDA_cam_" + std::to_string(i);
    w.width = c.width;
    w.height = c.height;
    auto t0 = std::chrono::steady_clock::now();
    int st = bvhgb_trace_image(s.cudaBVH.nodes, s.cudaBVH.numNodes, s.root, reinterpret_cast<const float *>(s.rawMesh.vert),
                               reinterpret_cast<const uint32_t *>(s.rawMesh.faces), &cam, &tc, img, hits, nullptr);
    if (st == BVHGB_OK) st = bvhgb_device_sync();
    w.ns = std::chrono::duration<double, std::nano>(std::chrono::steady_clock::now() - t0).count();
    if (st == BVHGB_OK) {
      w.pixels.resize(npx);
      w.hits.resize(npx);
      if (cudaMemcpy(w.pixels.data(), img, npx * sizeof(bvhgb_pixel), cudaMemcpyDeviceToHost) != cudaSuccess ||
          cudaMemcpy(w.hits.data(), hits, npx * sizeof(bvhgb_hit), cudaMemcpyDeviceToHost) != cudaSuccess)
        st = BVHGB_CUDA_ERROR;
    }
    cudaFree(img);
    cudaFree(hits);
    if (st) return from_status(st);
    s.work.push_back(std::move(w));
  }
  return ErrorCode::OK;
}

ErrorCode Validate::runImpl(State &s) {
  const auto &b = s.bvh;
  const size_t n = b.size();
  if (n == 0) return ErrorCode::OK;
  uint64_t tree = 0, box = 0, strict = 0, area = 0, tris = 0;
  // checkTree: parent links, left/right flags, distinct children, levels, orphans.
  std::vector<uint8_t> seen(n, 0);
  std::vector<std::pair<uint32_t, uint32_t>> st{{s.root, 0u}};
  if (b[s.root].parent != s.root) tree++;
  uint32_t maxLevel = 0;
  while (!st.empty()) {
    auto [x, lvl] = st.back();
    st.pop_back();
    if (x >= n || seen[x]) {
      tree++;
      continue;
    }
    seen[x] = 1;
    if (b[x].level != lvl) tree++;
    if (lvl > maxLevel) maxLevel = lvl;
    if (x != s.root && b[x].parent < n) {
      const auto &p = b[b[x].parent];
      if (b[x].isLeft ? p.left != x : p.right != x) tree++;
    }
    if (!b[x].isLeafFlag) {
      if (b[x].left == b[x].right || b[x].left == x || b[x].right == x || b[x].left >= n || b[x].right >= n) {
        tree++;
        continue;
      }
      if (b[b[x].left].parent != x) tree++;
      if (b[b[x].right].parent != x) tree++;
      st.push_back({b[x].right, lvl + 1});
      st.push_back({b[x].left, lvl + 1});
    }
  }
  for (size_t i = 0; i < n; ++i) tree += seen[i] ? 0 : 1;
  if (maxLevel != s.maxLevel) tree++;
  // checkBBoxes / checkBBoxesStrict / checkSurfaceArea
  for (size_t i = 0; i < n; ++i) {
    const auto &x = b[i];
    const auto &bb = x.bbox.minMax;
    const float dx = bb[1].x - bb[0].x, dy = bb[1].y - bb[0].y, dz = bb[1].z - bb[0].z;
    float xy = dx * dy, xz = dx * dz, yz = dy * dz;
    float sa = xy + xz;
    sa = sa + yz;
    sa = 2.0f * sa;
    if (!(std::fabs(x.surfaceArea - sa) < 0.000001f)) area++;
    if (x.isLeafFlag || x.left >= n || x.right >= n) continue;
    const auto &l = b[x.left].bbox.minMax, &r = b[x.right].bbox.minMax;
    bool e = !(bb[0].x <= l[0].x && bb[0].y <= l[0].y && bb[0].z <= l[0].z && bb[1].x >= l[1].x && bb[1].y >= l[1].y &&
               bb[1].z >= l[1].z && bb[0].x <= r[0].x && bb[0].y <= r[0].y && bb[0].z <= r[0].z && bb[1].x >= r[1].x &&
               bb[1].y >= r[1].y && bb[1].z >= r[1].z);
    bool es = !(bb[0].x == std::fmin(l[0].x, r[0].x) && bb[0].y == std::fmin(l[0].y, r[0].y) &&
                bb[0].z == std::fmin(l[0].z, r[0].z) && bb[1].x == std::fmax(l[1].x, r[1].x) &&
                bb[1].y == std::fmax(l[1].y, r[1].y) && bb[1].z == std::fmax(l[1].z, r[1].z));
    box += e;
    strict += es;
  }
  // checkTris
  const size_t nf = s.faces.size() / 3;
  std::vector<uint8_t> cov(nf, 0);
  for (size_t i = 0; i < n; ++i) {
    const auto &x = b[i];
    if (!x.isLeafFlag) continue;
    bool e = false;
    for (uint64_t f = x.left; f < (uint64_t)x.left + x.right; ++f) {
      if (f >= nf) {
        e = true;
        continue;
      }
      cov[f] = 1;
      for (int v = 0; v < 3; ++v) {
        const float *p = &s.vert[3ull * s.faces[3 * f + v]];
        const auto &bb = x.bbox.minMax;
        if (!(bb[0].x <= p[0] && bb[0].y <= p[1] && bb[0].z <= p[2] && bb[1].x >= p[0] && bb[1].y >= p[1] && bb[1].z >= p[2]))
          e = true;
      }
    }
    tris += e;
  }
  for (size_t f = 0; f < nf; ++f) tris += cov[f] ? 0 : 1;
  const uint64_t total = tree + box + strict + area + tris;
  if (total)
    error("validate: " + std::to_string(tree) + " tree, " + std::to_string(box) + " bbox, " + std::to_string(strict) +
          " strict bbox, " + std::to_string(area) + " surface area, " + std::to_string(tris) + " triangle errors");
  return total ? ErrorCode::WARNING : ErrorCode::OK;
}

const std::vector<std::string> &command_names() {
  static const std::vector<std::string> names = {"load",     "generate",  "camImport", "BVHExport",    "BVHImport",
                                                 "writeImg", "writeData", "copyToGPU", "copyToHost",   "LBVH",
                                                 "bittner13GPU", "CUDATracer", "status", "validate", "sleep"};
  return names;
}

CommandPtr command_from_string(const std::string &n) {
  if (n == "load") return std::make_shared<Load>();
  if (n == "generate") return std::make_shared<Generate>();
  if (n == "camImport") return std::make_shared<CamImport>();
  if (n == "BVHExport") return std::make_shared<BVHExport>();
  if (n == "BVHImport") return std::make_shared<BVHImport>();
  if (n == "writeImg") return std::make_shared<WriteImg>();
  if (n == "writeData") return std::make_shared<WriteData>();
  if (n == "copyToGPU") return std::make_shared<CopyToGPU>();
  if (n == "copyToHost") return std::make_shared<CopyToHost>();
  if (n == "LBVH") return std::make_shared<LBVH>();
  if (n == "bittner13GPU") return std::make_shared<Bittner13GPU>();
  if (n == "CUDATracer") return std::make_shared<CUDATracer>();
  if (n == "status") return std::make_shared<Status>();
  if (n == "validate") return std::make_shared<Validate>();
  if (n == "sleep") return std::make_shared<Sleep>();
  return nullptr;
}

void Config::fromJSON(const Json &j) {
  if (j.contains("baseConfig")) {
    const Json &b = j.at("baseConfig");
    name = b.value("name", name);
    verbose = b.value("verbose", verbose);
    basePath = b.value("basePath", basePath);
    if (b.contains("input") && b.at("input").is_array()) {
      input.clear();
      for (const Json &i : b.at("input").as_array())
        if (i.is_string()) input.push_back(i.as_string());
    }
  }
  if (!j.contains("commands") || !j.at("commands").is_array()) return;
  for (const Json &c : j.at("commands").as_array()) {
    const std::string n = c.at("cmd").as_string();
    CommandPtr cmd = command_from_string(n);
    if (!cmd) {
      warn("Command '" + n + "' not found");
      continue;
    }
    cmd->fromJSON(c.contains("options") ? c.at("options") : Json::object());
    commands.push_back(cmd);
  }
}

Json Config::toJSON() const {
  Json base = Json::object();
  base["name"] = name;
  base["verbose"] = verbose;
  base["basePath"] = basePath;
  Json in = Json::array();
  for (const auto &i : input) in.push_back(i);
  base["input"] = in;
  Json cmds = Json::array();
  for (const auto &c : commands) {
    Json e = Json::object();
    e["cmd"] = c->name();
    Json o = c->toJSON();
    if (o.size()) e["options"] = o;
    cmds.push_back(e);
  }
  Json out = Json::object();
  out["baseConfig"] = base;
  out["commands"] = cmds;
  return out;
}

int run_config_file(const std::string &path, std::string *log) {
  g_log = log;
  std::string text;
  if (!read_file(path, text)) {
    error("cannot read " + path);
    return 2;
  }
  Config cfg;
  try {
    cfg.fromJSON(Json::parse(text));
  } catch (const JsonError &e) {
    error(std::string("JSON exception: ") + e.what());
    return 2;
  }
  {
    std::ofstream f(path, std::ios::trunc);  // the config is rewritten with its defaults filled in
    f << cfg.toJSON().dump(2);
  }
  g_verbose = cfg.verbose;
  int worst = 0;
  for (const auto &in : cfg.input) {
    info("Processing " + in);
    State s;
    s.input = in;
    s.basePath = cfg.basePath;
    s.name = cfg.name;
    for (auto &c : cfg.commands) {
      ErrorCode r = c->run(s);
      if (r != ErrorCode::OK && r != ErrorCode::WARNING) {
        worst = (int)r;
        break;
      }
    }
  }
  g_log = nullptr;
  return worst;
}

}  // namespace bvhgb::host

// C entry points of the command layer.
extern "C" BVHGB_API int bvhgb_run_config(const char *path) {
  if (!path) return BVHGB_INVALID_ARGUMENT;
  return bvhgb::host::run_config_file(path);
}

extern "C" BVHGB_API int bvhgb_cli_main(int argc, char **argv) {
  using namespace bvhgb::host;
  std::vector<std::string> args(argv + 1, argv + argc);
  auto usage = []() {
    std::printf(
        "Options:\n"
        "  help               -- display this help message\n"
        "  run CFG            -- run BVHTest with configuration file CFG\n"
        "  list               -- list all commands and exit\n"
        "  generate FILE CMDs -- generate config file with commands CMDs (use - for stdout)\n");
    return 0;
  };
  if (args.empty()) return usage();
  for (size_t i = 0; i < args.size(); ++i) {
    const std::string &a = args[i];
    if (a == "list") {
      std::printf("Commands:\n");
      for (const auto &n : command_names()) std::printf("  - %-16s -- %s\n", n.c_str(), command_from_string(n)->desc().c_str());
      return 0;
    }
    if (a == "generate") {
      if (i + 1 >= args.size()) return usage();
      Config cfg;
      for (size_t k = i + 2; k < args.size(); ++k) {
        auto c = command_from_string(args[k]);
        if (!c) {
          std::fprintf(stderr, "Command '%s' not found\n", args[k].c_str());
          return 2;
        }
        cfg.commands.push_back(c);
      }
      const std::string text = cfg.toJSON().dump(2);
      if (args[i + 1] == "-") {
        std::printf("%s\n", text.c_str());
      } else {
        std::ofstream f(args[i + 1], std::ios::trunc);
        if (!f) return 1;
        f << text;
      }
      return 0;
    }
    if (a == "run") {
      if (++i >= args.size()) {
        std::fprintf(stderr, "Argument required for 'run'\n");
        return 1;
      }
      if (run_config_file(args[i]) != 0) return 2;
      continue;
    }
    return usage();
  }
  return 0;
}
