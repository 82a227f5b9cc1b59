// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY (the oracle's "reference" arm).
//
// Drives the reference simulator's own, unmodified step functions
// (src/simulation.cpp, src/interaction.cpp, src/postprocessing.cpp,
// src/mathFun.cpp, src/configuration.cpp of MD_Sim_Wolfschwenger) on injected
// particle states with a fixed time step, and dumps every intermediate array
// at full FP64 precision.  Nothing in the product links or loads this file;
// it is compiled by oracle/build_ref.sh into oracle/_ref/ and used only to
// pin the C restatement (oracle/md_oracle.c) and to write tests/golden/.
//
// Mechanism (no reference source is copied):
//   * the reference's simulation.cpp is #included with its `main` renamed, so
//     its file-static state (workVar, buffer, intCoeff, outputVar, params) and
//     its global RNG are reachable from this translation unit;
//   * `private` is mapped to `public` while configuration.h is parsed, so the
//     harness can override values the reference cannot express (particle
//     count that is not npDim^3, viscosity, per-particle radii) after the
//     singleton has parsed ../configuration.ini (configuration.cpp:6);
//   * fixed dt: absTol is set to +huge so AdjustTimeStep
//     (simulation.cpp:912-951) accepts every step, and deltaT is reset to
//     the fixed value before every step (the reference's own loop,
//     simulation.cpp:466-520, would otherwise let it grow).
//
// I/O: argv[1] = input file, argv[2] = output file (formats: oracle/ref_io.py);
// optional argv[3] = a directory where, after the last step, the reference's
// own writers put its text outputs (data.txt, coords.txt with two frames,
// dtMean/P/MSD .txt, mz.txt, t.txt), as RunSimulation would.
// The working directory must have ../configuration.ini (configuration.cpp:6).

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <set>
#include <unistd.h>
#include <string>
#include <vector>
#include <Eigen/Dense>
#include <EigenRand/EigenRand>

#define private public
#include "configuration.h"
#undef private

#define main md_reference_main_unused
#include "simulation.cpp"
#undef main

namespace {

struct In {
  int64_t n = 0, nsteps = 0, dump_level = 1, ewald_search = 0;
  int64_t has_radii = 0, has_pos = 0, has_orient = 0, adaptive = 0;
  double dt = 1e-12, alpha = 0, rc = 0, kc = 0, vis = 0;
  std::vector<double> rmag, pos, mm, ea;
};

bool rd(FILE* f, void* p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

void put(FILE* f, const double* p, size_t n) { fwrite(p, sizeof(double), n, f); }
void put1(FILE* f, double v) { fwrite(&v, sizeof(double), 1, f); }
// Eigen ArrayXXd (N x 3) is column-major: x[0..N), y[0..N), z[0..N).
void putArr(FILE* f, const ArrayXXd& a) { put(f, a.data(), (size_t)a.size()); }

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: ref_harness <in.bin> <out.bin>\n");
    return 2;
  }
  FILE* fi = fopen(argv[1], "rb");
  if (!fi) { perror("in"); return 2; }
  In in;
  int64_t hdr[8];
  double dh[5];
  if (!rd(fi, hdr, sizeof hdr) || !rd(fi, dh, sizeof dh)) { fprintf(stderr, "short header\n"); return 2; }
  // magic "MDREF": fixed step; "MDREG": one more header word, the adaptive flag
  if (hdr[0] != 0x4d44524546ll && hdr[0] != 0x4d44524547ll) { fprintf(stderr, "bad magic\n"); return 2; }
  if (hdr[0] == 0x4d44524547ll && !rd(fi, &in.adaptive, sizeof in.adaptive)) { fprintf(stderr, "short header\n"); return 2; }
  in.n = hdr[1]; in.nsteps = hdr[2]; in.dump_level = hdr[3]; in.ewald_search = hdr[4];
  in.has_radii = hdr[5]; in.has_pos = hdr[6]; in.has_orient = hdr[7];
  in.dt = dh[0]; in.alpha = dh[1]; in.rc = dh[2]; in.kc = dh[3]; in.vis = dh[4];
  const int64_t n = in.n;
  if (in.has_radii) { in.rmag.resize(n); if (!rd(fi, in.rmag.data(), 8 * n)) return 2; }
  if (in.has_pos) { in.pos.resize(3 * n); if (!rd(fi, in.pos.data(), 24 * n)) return 2; }
  if (in.has_orient) {
    in.mm.resize(3 * n); in.ea.resize(3 * n);
    if (!rd(fi, in.mm.data(), 24 * n) || !rd(fi, in.ea.data(), 24 * n)) return 2;
  }
  fclose(fi);

  if (config->reader.ParseError() != 0) { fprintf(stderr, "configuration.ini not parsed\n"); return 3; }
  // Extensions the reference cannot express (values only; formulas unchanged).
  config->numbPart_ = (int)n;
  if (in.vis > 0) config->vis_ = in.vis;
  // fixed step: every step accepted; adaptive: the INI's absTol and the
  // reference's own step control, with in.dt as the first trial step
  if (!in.adaptive) config->absTol_ = 1e300;

  WorkingVar_S* pW = &workVar;
  // particle properties: the reference's own routine, or injected radii
  // followed by the same derived-property formulas (simulation.cpp:204-210).
  InitParticleProps(&pW->partProp);
  if (in.has_radii) {
    PartProps_S* p = &pW->partProp;
    for (int64_t i = 0; i < n; i++) p->rMag(i) = in.rmag[i];
    if (config->getEnableCoatingPot()) {
      for (int64_t i = 0; i < n; i++) {
        double dH = IntegralEffDiameter(2 * p->rMag(i));
        p->rHydr(i) = dH >= 2 * p->rMag(i) ? dH / 2.0 : p->rMag(i);
      }
    } else {
      p->rHydr = p->rMag + config->getDShell();
    }
    p->volMag = 4.0 / 3.0 * config->getMyPi() * p->rMag.pow(3.0);
    p->volHydr = 4.0 / 3.0 * config->getMyPi() * p->rHydr.pow(3.0);
    p->magMom = config->getSatMag() * p->volMag;
    p->zetaRot = 8.0 * config->getMyPi() * config->getVis() * p->rHydr.pow(3.0);
    p->zetaTrans = 6.0 * config->getMyPi() * config->getVis() * p->rHydr;
    p->velEaConst1 = 2.0 * config->getAnisEn() * (p->volMag / p->zetaRot);
    p->velEaConst2 = p->zetaRot.cwiseInverse();
  }
  params.lBox = pow(pW->partProp.volHydr.sum() / config->getVolFrac(), 1.0 / 3.0);
  params.volBox = pow(params.lBox, 3.0);
  params.transOutput = false;

  // Initial coordinates: the reference's RSA + orientation draw, then overrides.
  InitCoordsFromSketch(pW, &params);
  if (in.has_pos)
    for (int64_t i = 0; i < 3 * n; i++) pW->coordsTrans.pos.data()[i] = in.pos[i];
  if (in.has_orient)
    for (int64_t i = 0; i < 3 * n; i++) {
      pW->coordsRot.posMm.data()[i] = in.mm[i];
      pW->coordsRot.posEa.data()[i] = in.ea[i];
    }

  InitIntCoeff(&intCoeff);
  InitBuffers(&buffer);
  InitCutOffSR(&params, &pW->partProp);
  int64_t maxPairs = n * (n - 1) / 2;
  pW->intLists.intVecsCoords.resize(maxPairs, 3);
  pW->intLists.intVecsLen.resize(maxPairs);
  pW->intLists.intPairs.resize(2 * maxPairs);
  pW->intLists.intRangeSR.resize(maxPairs);
  pW->intLists.intRangeSR.setConstant(false);  // first step: the intended cutoff
  pW->extFluxDens.resize(n, 3); pW->extFluxDens.setZero();
  pW->demagFluxDens.resize(n, 3); pW->demagFluxDens.setZero();
  pW->intForce.resize(n, 3); pW->intForce.setZero();
  pW->thermTorque.resize(n, 3); pW->thermField.resize(n, 3); pW->thermForce.resize(n, 3);

  if (in.ewald_search) {
    CompEwaldParams(pW, &buffer, &params);
  } else {
    params.alpha = in.alpha;
    params.rCutLR = in.rc;
    params.nCutLR = in.kc;
  }
  InitEwaldConst(&params, &buffer);
  outputVar.posRef = pW->coordsTrans.pos;
  outputVar.truePos = pW->coordsTrans.pos;

  FILE* fo = fopen(argv[2], "wb");
  if (!fo) { perror("out"); return 2; }
  put1(fo, params.lBox); put1(fo, params.alpha); put1(fo, params.rCutLR); put1(fo, params.nCutLR);
  put1(fo, params.rCutSR);
  put1(fo, config->getVis());
  put(fo, pW->partProp.rMag.data(), n);
  put(fo, pW->partProp.rHydr.data(), n);
  putArr(fo, pW->coordsTrans.pos);
  putArr(fo, pW->coordsRot.posMm);
  putArr(fo, pW->coordsRot.posEa);

  double tInt = 0, deltaT = in.dt, deltaTused = in.dt;
  timespec t0, t1;
  double elapsed = 0;
  for (int64_t s = 0; s < in.nsteps; s++) {
    if (!in.adaptive) deltaT = in.dt;
    if (in.adaptive) put1(fo, deltaT);  // the trial step DefThermFluct scales the noise with
    clock_gettime(CLOCK_MONOTONIC, &t0);
    DefExtField(&pW->extFluxDens, tInt);
    DefThermFluct(pW, &buffer.buffer1d, deltaT);
    EvalSinCos(pW, &buffer, &params);
    CompInteractions(pW, &buffer, &params, &outputVar);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    elapsed += (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    if (in.dump_level >= 1) {
      putArr(fo, pW->demagFluxDens);   // B after CompInteractions
      putArr(fo, pW->intForce);        // F incl. thermal force
      putArr(fo, pW->thermTorque);
      putArr(fo, pW->thermField);
      putArr(fo, pW->thermForce);
      putArr(fo, pW->coordsTrans.pos); // after the in-place overlap push
      put1(fo, (double)pW->intLists.pairs);
    }
    clock_gettime(CLOCK_MONOTONIC, &t0);
    IntegrationRot(pW, &intCoeff, &buffer, &params, &deltaT, &deltaTused);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    elapsed += (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    if (in.dump_level >= 1) putArr(fo, pW->demagFluxDens);  // B at the Heun predictor
    clock_gettime(CLOCK_MONOTONIC, &t0);
    IntegrationTrans(pW, &buffer, &params, deltaTused);
    ApplyBoundaryCondArr(&pW->coordsTrans.pos, &buffer.buffer3d, &params);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    elapsed += (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    EvalTransCoeffs(pW, &buffer, &outputVar, &params);
    double mz = pW->coordsRot.posMm.col(2).mean();
    outputVar.t.push_back(tInt);
    outputVar.mz.push_back(mz);
    if (in.dump_level >= 1) {
      putArr(fo, pW->coordsTrans.pos);
      putArr(fo, pW->coordsRot.posMm);
      putArr(fo, pW->coordsRot.posEa);
    }
    if (in.dump_level >= 0) {
      double obs[8] = {tInt, mz, outputVar.MSDx.back(), outputVar.MSDy.back(), outputVar.MSDz.back(),
                       outputVar.PxyVec.back(), outputVar.PxzVec.back(), outputVar.PyzVec.back()};
      put(fo, obs, 8);
    }
    if (in.adaptive) put1(fo, deltaTused);
    tInt += deltaTused;
  }
  putArr(fo, pW->coordsTrans.pos);
  putArr(fo, pW->coordsRot.posMm);
  putArr(fo, pW->coordsRot.posEa);
  put1(fo, elapsed);
  fclose(fo);
  if (argc > 3) {
    if (chdir(argv[3]) != 0) { perror("txt dir"); return 2; }
    WriteData2TXT(pW, &params, "data.txt");
    WriteCoords2TXT(pW, "coords.txt", 0.0);
    WriteCoords2TXT(pW, "coords.txt", tInt);
    ExportDiffVis(&outputVar, tInt, (int)in.nsteps);
    saveData("mz.txt", Map<VectorXd, Unaligned>(outputVar.mz.data(), outputVar.mz.size()), 0);
    saveData("t.txt", Map<VectorXd, Unaligned>(outputVar.t.data(), outputVar.t.size()), 0);
  }
  return 0;
}
