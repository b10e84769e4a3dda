// Dump harness around the reference's own CPU implementation of the coupled
// solid-fluid step. Test infrastructure only: it is compiled by
// oracle/Makefile against the unmodified reference sources and is used to
// (1) pin the C restatement in oracle/esf_oracle.c and (2) write the golden
// fixtures under tests/golden/. Nothing in the product links it.
//
// It replaces the GLUT application of projects/rubberBall/main.cpp:30-243
// with a headless loop that keeps that file's set-up order
// (APPLICATION::init :63-97, addSolids :99-160) and its frame/substep loop
// (APPLICATION::step :174-204), and writes every intermediate field as .npy.
//
// usage: ref_harness <cfg> <outdir> <frames> [--noise <file.npy-raw f64 X^3*3>]
//                    [--dump-every k] [--no-dump] [--full-every k] [--frame-restart dir]
//
// --frame-restart dir: after the last step, COUPLED_INTEGRATOR_3D::writeFrame
// (frame 0, debug) writes the state into dir; a second integrator built the
// same way reads it back (readFrame), writes it again as frame 1, and takes
// one step; its state after the read and after that step is dumped with the
// prefixes "r0." and "r1.", and the step's log line goes to log_restart.jsonl.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>
#include <sys/stat.h>
#include <sys/time.h>
#include <unistd.h>
#include <Eigen/Dense>
#include <Eigen/Sparse>
#include <Eigen/Geometry>
#include <Eigen/SVD>
#include <Eigen/IterativeLinearSolvers>
#include <Eigen/SparseLU>
#if USING_OPENMP_HARNESS
#include <omp.h>
#endif

// Private access to the integrator's and solid's state for dumping.
#define private public
#define protected public
#include <SETTINGS.h>
#include <integrator/COUPLED_INTEGRATOR_3D.h>
#include <integrator/DEFOR_SOLID_3D.h>
#include <util/SIMPLE_PARSER.h>
#include <util/TIMING_BREAKDOWN.h>
#undef private
#undef protected

// The warm-started pressure solution is a function-local static of
// COUPLED_INTEGRATOR_3D::pcrImplicitSolve (COUPLED_INTEGRATOR_3D.cpp:712).
// oracle/Makefile makes its symbol global in the object file so it can be read.
extern VECTOR ref_lambda1 __asm__("_ZZN21COUPLED_INTEGRATOR_3D16pcrImplicitSolveEvE7lambda1");

static double now_s() {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}

// ---------------------------------------------------------------- npy writer
static void write_npy(const std::string& path, const char* descr,
                      const std::vector<long>& shape, const void* data,
                      size_t bytes) {
  std::ostringstream hdr;
  hdr << "{'descr': '" << descr << "', 'fortran_order': False, 'shape': (";
  for (size_t i = 0; i < shape.size(); i++) {
    hdr << shape[i];
    if (shape.size() == 1 || i + 1 < shape.size()) hdr << ",";
    if (i + 1 < shape.size()) hdr << " ";
  }
  hdr << "), }";
  std::string h = hdr.str();
  size_t total = 10 + h.size() + 1;
  size_t pad = (64 - total % 64) % 64;
  h += std::string(pad, ' ');
  h += "\n";
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) {
    fprintf(stderr, "cannot write %s\n", path.c_str());
    exit(2);
  }
  const char magic[] = "\x93NUMPY\x01\x00";
  fwrite(magic, 1, 8, f);
  unsigned short hl = (unsigned short)h.size();
  fwrite(&hl, 2, 1, f);
  fwrite(h.data(), 1, h.size(), f);
  if (bytes) fwrite(data, 1, bytes, f);
  fclose(f);
}

struct Dumper {
  std::string dir;
  std::string prefix;
  void f64(const std::string& name, const double* p, long n,
           std::vector<long> shape = {}) {
    if (shape.empty()) shape = {n};
    write_npy(dir + "/" + prefix + name + ".npy", "<f8", shape, p, n * 8);
  }
  void vec(const std::string& name, const VECTOR& v) {
    f64(name, v.data(), v.size());
  }
  void i32(const std::string& name, const int* p, long n) {
    write_npy(dir + "/" + prefix + name + ".npy", "<i4", {n}, p, n * 4);
  }
  void i8(const std::string& name, const char* p, long n) {
    write_npy(dir + "/" + prefix + name + ".npy", "|i1", {n}, p, n);
  }
  void field(const std::string& name, const FIELD_3Df& f) {
    f64(name, f.data().data(), f.totalCells());
  }
  void vfield(const std::string& name, const VEC3F_FIELD_3D& f) {
    std::vector<double> tmp(f.totalCells() * 3);
    for (int i = 0; i < f.totalCells(); i++)
      for (int d = 0; d < 3; d++) tmp[i * 3 + d] = f[i][d];
    f64(name, tmp.data(), tmp.size(), {(long)f.totalCells(), 3});
  }
  void spmat(const std::string& name, SpMat m) {
    m.makeCompressed();
    std::vector<int> outer(m.outerIndexPtr(), m.outerIndexPtr() + m.rows() + 1);
    std::vector<int> inner(m.innerIndexPtr(), m.innerIndexPtr() + m.nonZeros());
    std::vector<double> val(m.valuePtr(), m.valuePtr() + m.nonZeros());
    i32(name + ".indptr", outer.data(), outer.size());
    i32(name + ".indices", inner.data(), inner.size());
    f64(name + ".data", val.data(), val.size());
  }
};

// the rotation each solid was set up with (main.cpp:131-136 builds it through
// Eigen quaternions), dumped so that other implementations can take it as is
static std::vector<MATRIX3> harnessRotations;

static void dump_state(Dumper& d, COUPLED_INTEGRATOR_3D* I, bool full) {
  d.vfield("velocity", I->_velocity);
  d.field("intensity", I->_intensity);
  d.field("solidMass", I->_solidMass);
  d.field("nodeSolidVolumeFraction", I->_nodeSolidVolumeFraction);
  if (!I->_gridIdxToSolutionIdx.empty())
    d.i32("gridIdxToSolutionIdx", I->_gridIdxToSolutionIdx.data(),
          I->_gridIdxToSolutionIdx.size());
  d.i32("gridIdxToSolidIdx", I->_gridIdxToSolidIdx.data(),
        I->_gridIdxToSolidIdx.size());
  d.vec("lambda1", ref_lambda1);
  if (full) {
    d.vec("nzMassVecInv", I->_nzMassVecInv);
    d.vec("JMInvJTDiag", I->_JMInvJTDiag);
    d.vec("divergenceConstraintsRHS", I->_divergenceConstraintsRHS);
    d.vec("velocityAtDt0", I->_velocityAtDt0);
    d.vec("velocityAtDt1", I->_velocityAtDt1);
    d.vec("pressureCorrection", I->_pressureCorrection);
    d.vec("unitForce", I->_unitForce);
    d.vec("mv", I->_mv);
    d.vec("solidUnitForce", I->_solidUnitForce);
    d.vec("solidMv", I->_solidMv);
    d.vec("dampedSolidMassVec", I->_dampedSolidMassVec);
    d.vec("solidVelocityAtDt0", I->_solidVelocityAtDt0);
    d.vec("solidPressureCorrection", I->_solidPressureCorrection);
    if (I->_systemMatrix.rows() > 0) d.spmat("systemMatrix", I->_systemMatrix);
    if (I->_velocityAtDt0.size() > 0) {
      VECTOR b1 = I->_divergenceConstraintJacobian * I->_velocityAtDt0 -
                  I->_divergenceConstraintsRHS;
      d.vec("b1", b1);
    }
  }
  for (size_t s = 0; s < I->_solids.size(); s++) {
    DEFOR_SOLID_3D* S = I->_solids[s];
    Dumper ds = d;
    ds.prefix = d.prefix + "solid" + std::to_string(s) + ".";
    ds.vfield("u", S->_u);
    ds.vfield("X", S->_X);
    ds.vfield("velocity", S->_velocity);
    ds.vfield("vecWorkspace", S->_vecWorkspace);
    ds.field("mass", S->_mass);
    ds.field("phi", S->_phi);
    ds.field("detFInv", S->_detFInv);
    ds.i8("valid", S->_valid.data().data(), S->_valid.totalCells());
    ds.vec("quarterVolumeFractions", S->_quarterVolumeFractions);
    int box[12] = {S->_xmin,        S->_ymin,        S->_zmin,
                   S->_xmax,        S->_ymax,        S->_zmax,
                   S->_tightMin[0], S->_tightMin[1], S->_tightMin[2],
                   S->_tightMax[0], S->_tightMax[1], S->_tightMax[2]};
    ds.i32("boxes", box, 12);
    if (s < harnessRotations.size()) {
      double rm[9];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) rm[i * 3 + j] = harnessRotations[s](i, j);
      ds.f64("rotation", rm, 9);
    }
    long np = S->_materialParticles.size();
    std::vector<double> pp(np * 10);
    for (long i = 0; i < np; i++) {
      const PARTICLE& p = S->_materialParticles[i];
      for (int k = 0; k < 3; k++) {
        pp[i * 10 + k] = p.pos[k];
        pp[i * 10 + 3 + k] = p.velocity[k];
        pp[i * 10 + 6 + k] = p.restPos[k];
      }
      pp[i * 10 + 9] = p.mass;
    }
    ds.f64("particles", pp.data(), pp.size(), {np, 10});
    std::vector<VEC3F>& verts = S->_surfaceMesh->vertices;
    std::vector<double> vv(verts.size() * 3);
    for (size_t i = 0; i < verts.size(); i++)
      for (int k = 0; k < 3; k++) vv[i * 3 + k] = verts[i][k];
    ds.f64("meshVertices", vv.data(), vv.size(), {(long)verts.size(), 3});
    if (S->_isPlastic) {
      // inverse plastic deformation gradient on the material grid, row-major
      const MATRIX3_FIELD_3D& F = S->_FpInv;
      std::vector<double> fp((size_t)F._totalCells * 9);
      for (int c = 0; c < F._totalCells; c++)
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) fp[(size_t)c * 9 + i * 3 + j] = F._data[c](i, j);
      ds.f64("FpInv", fp.data(), fp.size(), {(long)F._totalCells, 3, 3});
      double hdr[7] = {(double)F._xRes, (double)F._yRes, (double)F._zRes, F._dh,
                       F._origin[0], F._origin[1], F._origin[2]};
      ds.f64("FpInvGrid", hdr, 7);
    }
  }
}

// APPLICATION::init (projects/rubberBall/main.cpp:63-97) and addSolids
// (:99-160), headless: a new integrator with the cfg's solids, initialised.
static COUPLED_INTEGRATOR_3D* build_integrator() {
  // APPLICATION::init (projects/rubberBall/main.cpp:63-97), headless.
  int xRes = SIMPLE_PARSER::getInt("xRes", 100);
  int yRes = SIMPLE_PARSER::getInt("yRes", 100);
  int zRes = SIMPLE_PARSER::getInt("zRes", 100);
  Real dh = SIMPLE_PARSER::getFloat("dh", 0.01);
  VEC3F origin = SIMPLE_PARSER::getVEC3F("origin", VEC3F(0, 0, 0));
  COUPLED_INTEGRATOR_3D* integrator =
      new COUPLED_INTEGRATOR_3D(xRes, yRes, zRes, dh, origin);

  // addSolids (main.cpp:99-160). The DT-Grid rest SDF is only read by
  // solid-solid contact (DEFOR_SOLID_3D.cpp:969-995), so it is loaded only
  // when the scene has more than one solid.
  int numberOfSolids = SIMPLE_PARSER::getInt("number of solids", 1);
  for (int i = 0; i < numberOfSolids; i++) {
    std::string index = std::to_string(i);
    std::string meshPath = SIMPLE_PARSER::getString("solid path " + index, "");
    meshPath += SIMPLE_PARSER::getString("solid name " + index, "");
    FIELD_3Df restMass;
    restMass.readGz(meshPath + ".mass");
    DEFOR_SOLID_3D* solid = new DEFOR_SOLID_3D(xRes, yRes, zRes, dh, origin,
                                               restMass);
    Real lambda = SIMPLE_PARSER::getFloat("material lambda " + index, 100);
    Real mu = SIMPLE_PARSER::getFloat("material mu " + index, 100);
    solid->setMaterial(lambda, mu);
    solid->setMassDensity(
        SIMPLE_PARSER::getFloat("solid mass density " + index, 1));
    Real plasticYield =
        SIMPLE_PARSER::getFloat("solid plastic yield " + index, -1);
    if (plasticYield > 0) solid->setPlasticYield(plasticYield);
    VEC3F translation =
        SIMPLE_PARSER::getVEC3F("solid translation " + index, VEC3F(0, 0, 0));
    VEC3F scaling =
        SIMPLE_PARSER::getVEC3F("solid scaling " + index, VEC3F(1, 1, 1));
    VEC3F rotation =
        SIMPLE_PARSER::getVEC3F("solid rotation " + index, VEC3F(0, 0, 0));
    MATRIX3 rot;
    rot = Eigen::AngleAxisd(rotation[0] * M_PI, VEC3F::UnitX()) *
          Eigen::AngleAxisd(rotation[1] * M_PI, VEC3F::UnitY()) *
          Eigen::AngleAxisd(rotation[2] * M_PI, VEC3F::UnitZ());
    solid->setInitialState(rot, translation, scaling);
    harnessRotations.push_back(rot);
    solid->setInitialVelocity(SIMPLE_PARSER::getVEC3F(
        "solid initial velocity " + index, VEC3F(0, 0, 0)));
    solid->loadSurfaceMesh(meshPath + ".obj");
    if (numberOfSolids > 1) solid->loadRestSDF(meshPath + ".svol");
    OBJ* surfaceMesh = solid->surfaceMesh();
    surfaceMesh->scale(scaling);
    surfaceMesh->transformMesh(rot);
    surfaceMesh->translateMesh(translation);
    integrator->addSolid(solid);
  }
  integrator->setFluidDensity(SIMPLE_PARSER::getFloat("fluid density", 1));
  integrator->setFluidViscocity(SIMPLE_PARSER::getFloat("fluid viscocity", 0));
  integrator->init();
  return integrator;
}

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr,
            "usage: %s <cfg> <outdir> <frames> [--noise file] [--dump-every k]"
            " [--no-dump] [--full-every k]\n",
            argv[0]);
    return 2;
  }
  std::string cfg = argv[1];
  std::string outdir = argv[2];
  int frames = atoi(argv[3]);
  std::string noiseFile;
  int dumpEvery = 1, fullEvery = 1;
  bool noDump = false;
  std::string restartDir, sdfQueryFile;
  double sdfQuerySafe = 0;
  for (int a = 4; a < argc; a++) {
    std::string s = argv[a];
    if (s == "--noise" && a + 1 < argc) noiseFile = argv[++a];
    else if (s == "--dump-every" && a + 1 < argc) dumpEvery = atoi(argv[++a]);
    else if (s == "--full-every" && a + 1 < argc) fullEvery = atoi(argv[++a]);
    else if (s == "--no-dump") noDump = true;
    else if (s == "--frame-restart" && a + 1 < argc) restartDir = argv[++a];
    else if (s == "--sdf-query" && a + 2 < argc) {
      sdfQueryFile = argv[++a];
      sdfQuerySafe = atof(argv[++a]);
    }
  }
  mkdir(outdir.c_str(), 0755);
  Eigen::initParallel();
  if (!SIMPLE_PARSER::parse(cfg)) return 3;

  double t0 = now_s();
  COUPLED_INTEGRATOR_3D* integrator = build_integrator();
  const int xRes = integrator->xRes(), yRes = integrator->yRes(), zRes = integrator->zRes();
  const Real dh = integrator->dh();

  Real carpetThickness = SIMPLE_PARSER::getFloat("smoke carpet thickness", 0.06);
  int carpetLayers = carpetThickness / dh;
  FIELD_3Df& intensity = integrator->intensity();
  for (int z = 1; z < zRes - 1; z++)
    for (int y = 1; y < carpetLayers; y++)
      for (int x = 1; x < xRes - 1; x++) intensity(x, y, z) = 0.8f;

  // Seeded fluid noise: added to the grid velocity at nodes without solid
  // mass. The file holds raw little-endian doubles, X*Y*Z*3.
  if (!noiseFile.empty()) {
    FILE* f = fopen(noiseFile.c_str(), "rb");
    if (!f) {
      fprintf(stderr, "cannot read %s\n", noiseFile.c_str());
      return 4;
    }
    long n = (long)xRes * yRes * zRes;
    std::vector<double> buf(n * 3);
    if (fread(buf.data(), 8, n * 3, f) != (size_t)(n * 3)) {
      fprintf(stderr, "short noise file\n");
      return 4;
    }
    fclose(f);
    for (long i = 0; i < n; i++)
      if (integrator->_solidMass[i] == 0)
        for (int d = 0; d < 3; d++) integrator->_velocity[i][d] += buf[i * 3 + d];
  }
  double tInit = now_s() - t0;

  // SPARSE_SDF::signedDistAndCurrentNormal of every solid with a rest SDF at
  // the rest points of the file (raw doubles, 3 per point), after init:
  // sdfq.solid<s>.npy holds n x 4 (distance, normal)
  if (!sdfQueryFile.empty()) {
    FILE* f = fopen(sdfQueryFile.c_str(), "rb");
    if (!f) return 4;
    std::vector<double> pts;
    double buf[3];
    while (fread(buf, 8, 3, f) == 3) pts.insert(pts.end(), buf, buf + 3);
    fclose(f);
    long n = (long)pts.size() / 3;
    Dumper dq;
    dq.dir = outdir;
    dq.prefix = "sdfq.";
    for (size_t si = 0; si < integrator->_solids.size(); si++) {
      SPARSE_SDF* sdf = integrator->_solids[si]->_restSDF;
      if (!sdf) continue;
      std::vector<double> res(n * 4);
      for (long i = 0; i < n; i++) {
        VEC3F p(pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]), normal(0, 0, 0);
        res[i * 4] = sdf->signedDistAndCurrentNormal(p, normal, sdfQuerySafe);
        for (int k = 0; k < 3; k++) res[i * 4 + 1 + k] = normal[k];
      }
      dq.f64(("solid" + std::to_string(si)).c_str(), res.data(), res.size(), {n, 4});
    }
  }

  Dumper d;
  d.dir = outdir;
  d.prefix = "s0.";
  if (!noDump) dump_state(d, integrator, false);

  // APPLICATION::step (main.cpp:174-204): one frame is a loop of substeps.
  FILE* log = fopen((outdir + "/log.jsonl").c_str(), "w");
  fprintf(log, "{\"init_s\": %.6f}\n", tInit);
  Real frameTimeStep = SIMPLE_PARSER::getFloat("dt", 0.005);
  int stepCount = 0;
  for (int frame = 0; frame < frames; frame++) {
    Real simTimeStep = 0;
    while (simTimeStep < frameTimeStep) {
      integrator->setMaxDt(frameTimeStep - simTimeStep);
      size_t n1 = integrator->_solver.numberOfIterations().size();
      size_t n2 = integrator->_divFreeSolver.numberOfIterations().size();
      double ts = now_s();
      Real energy = integrator->stepImplicit();
      double te = now_s() - ts;
      simTimeStep += integrator->dt();
      stepCount++;
      std::vector<int>& it1 = integrator->_solver.numberOfIterations();
      std::vector<int>& it2 = integrator->_divFreeSolver.numberOfIterations();
      fprintf(log,
              "{\"step\": %d, \"frame\": %d, \"dt\": %.17g, \"energy\": %.17g, "
              "\"seconds\": %.6f, \"solid_iters\": [",
              stepCount, frame, integrator->dt(), energy, te);
      for (size_t k = n1; k < it1.size(); k++)
        fprintf(log, "%s%d", k > n1 ? ", " : "", it1[k]);
      fprintf(log, "], \"pressure_iters\": [");
      for (size_t k = n2; k < it2.size(); k++)
        fprintf(log, "%s%d", k > n2 ? ", " : "", it2[k]);
      fprintf(log, "]}\n");
      fflush(log);
      if (!noDump && (stepCount % dumpEvery == 0)) {
        d.prefix = "s" + std::to_string(stepCount) + ".";
        dump_state(d, integrator, (stepCount % fullEvery) == 0);
      }
    }
  }
  fclose(log);
  if (!restartDir.empty()) {
    // COUPLED_INTEGRATOR_3D::writeFrame/readFrame take their directory from
    // the "data path" key (empty here), so the files go to the working directory
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return 5;
    mkdir(restartDir.c_str(), 0755);
    if (chdir(restartDir.c_str()) != 0) return 5;
    integrator->writeFrame(0, true);
    COUPLED_INTEGRATOR_3D* again = build_integrator();
    again->readFrame(0, true);
    again->writeFrame(1, true);
    if (chdir(cwd) != 0) return 5;
    Dumper dr;
    dr.dir = outdir;
    dr.prefix = "r0.";
    dump_state(dr, again, false);
    again->setMaxDt(frameTimeStep);
    size_t n1 = again->_solver.numberOfIterations().size();
    size_t n2 = again->_divFreeSolver.numberOfIterations().size();
    Real energy = again->stepImplicit();
    FILE* rl = fopen((outdir + "/log_restart.jsonl").c_str(), "w");
    std::vector<int>& it1 = again->_solver.numberOfIterations();
    std::vector<int>& it2 = again->_divFreeSolver.numberOfIterations();
    fprintf(rl, "{\"step\": 1, \"dt\": %.17g, \"energy\": %.17g, \"solid_iters\": [", again->dt(), energy);
    for (size_t k = n1; k < it1.size(); k++) fprintf(rl, "%s%d", k > n1 ? ", " : "", it1[k]);
    fprintf(rl, "], \"pressure_iters\": [");
    for (size_t k = n2; k < it2.size(); k++) fprintf(rl, "%s%d", k > n2 ? ", " : "", it2[k]);
    fprintf(rl, "]}\n");
    fclose(rl);
    dr.prefix = "r1.";
    dump_state(dr, again, false);
  }
  delete integrator;
  return 0;
}
