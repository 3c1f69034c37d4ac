// The reference's driver (src/BES.cpp:40-121) with the solve on the GPU: the reference's own
// Config, Mesh and Gas are built from the .besi file as in its main(), then SolverGpu runs
// the solve through libbes_gb300.so.  With --operators it instead evaluates the gradient,
// limiter and local time step of the freestream-initialised snapshot both with the
// reference's operator classes and with the GPU adapters, and prints their largest
// differences.
#include <cmath>
#include <cstring>

#include "GasPerfect.hpp"
#include "GradientGreenGauss.hpp"
#include "LimiterVenkatakrishnan.hpp"
#include "TimeStepCalculatorLocal.hpp"
#include "bes_reference_adapters.hpp"

int main(int argc, char* argv[]) {
  const bool ops = argc == 3 && std::strcmp(argv[1], "--operators") == 0;
  if (argc != 2 && !ops) {
    std::cout << "ERROR: usage: bes_driver [--operators] <file.besi>. Exiting..." << std::endl;
    return EXIT_FAILURE;
  }
  const std::string besi = argv[argc - 1];
  Config* config = new Config();
  Mesh* mesh = new Mesh();
  Gas* gas = new GasPerfect();
  config->initialize(besi);
  mesh->initialize(config);
  config->initializePostMesh(mesh);
  gas->initialize(config);
  std::cout << "reference objects built: " << mesh->getNumElement() << " cells" << std::endl;

  bes_ref::GpuPath gpu(besi);
  if (!ops) {
    bes_ref::SolverGpu solver(&gpu);
    solver.initialize(config, gas, mesh);
    solver.setUniversalInitialCondition(config->getFreestreamPrimitiveVariables(0));
    solver.solve();
  } else {
    // a freestream snapshot with a smooth perturbation, so that gradients and limiters are not
    // trivial
    SolutionSnapshot s;
    s.initialize(config, mesh, gas);
    const short nv = config->getNumConservedVariable();
    std::vector<double> U(5 * gpu.cells());
    gpu.check(bes_set_freestream_state(gpu.ctx()), "bes_set_freestream_state");
    gpu.check(bes_get_state(gpu.ctx(), U.data()), "bes_get_state");
    for (unsigned long i = 0; i < mesh->getNumElement(); ++i)
      for (short v = 0; v < nv; ++v)
        s.setConservedVariable(i, v, U[i * 5 + gpu.lib_var(v)] * (1.0 + 0.01 * std::sin(0.37 * i + v)));
    s.computeAllPrimitiveVariable();
    GradientGreenGauss gr;
    bes_ref::GradientGpu gg(&gpu);
    gr.initialize(config, mesh, CONSERVED);
    gg.initialize(config, mesh, CONSERVED);
    gr.computeGradient(&s);
    gg.computeGradient(&s);
    LimiterVenkatakrishnan lr;
    bes_ref::LimiterGpu lg(&gpu);
    lr.initialize(config, mesh, CONSERVED);
    lg.initialize(config, mesh, CONSERVED);
    lr.computeLimiterTerm(&s, &gr);
    lg.computeLimiterTerm(&s, &gg);
    TimeStepCalculatorLocal tr;
    bes_ref::TimeStepCalculatorGpu tg(&gpu, false);
    tr.initialize(config, gas, mesh);
    tg.initialize(config, gas, mesh);
    const double cfl = 0.8;
    tr.computeAllTimeStep(&s, cfl);
    tg.computeAllTimeStep(&s, cfl);
    double eg = 0, sg = 0, el = 0, et = 0, st = 0;
    for (unsigned long i = 0; i < mesh->getNumElement(); ++i) {
      for (short v = 0; v < nv; ++v) {
        for (short d = 0; d < mesh->getNumDim(); ++d) {
          eg = std::fmax(eg, std::fabs(gr.getGradient(i, v, d) - gg.getGradient(i, v, d)));
          sg = std::fmax(sg, std::fabs(gr.getGradient(i, v, d)));
        }
        el = std::fmax(el, std::fabs(lr.getLimiterValue(i, v) - lg.getLimiterValue(i, v)));
      }
      et = std::fmax(et, std::fabs(tr.getTimeStep(i) - tg.getTimeStep(i)));
      st = std::fmax(st, std::fabs(tr.getTimeStep(i)));
    }
    std::cout << "gradient max rel diff " << eg / sg << ", limiter max abs diff " << el
              << ", time step max rel diff " << et / st << std::endl;
  }
  delete gas;
  delete mesh;
  delete config;
  return EXIT_SUCCESS;
}
