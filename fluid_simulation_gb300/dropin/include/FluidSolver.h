// Drop-in for the reference's include/FluidSolver.h: the same classes and
// public methods, each step running on the GPU (fsgpu).  The solver's
// scratch memory lives with the domain's device state; the pool object
// keeps the sizes the reference validates against, including the
// reference's copy-constructor behaviour of keeping delta_x for delta_y
// (src/FluidSolver.cpp:56-62), so that validate() accepts and rejects the
// same domains.  Failures throw std::runtime_error, as the reference does.
#ifndef FLUID_SOLVER_H
#define FLUID_SOLVER_H

#include <FluidDomain.h>

#include "MathDefinitions.h"

class FluidSolverMemoryPool : public GridInterface
{
public:
    FluidSolverMemoryPool(int size_x, int size_y, MyFloat delta_x, MyFloat delta_y);
    FluidSolverMemoryPool(const FluidDomain& fluid_domain);
    FluidSolverMemoryPool(const FluidSolverMemoryPool& other);
    ~FluidSolverMemoryPool();
    void swapValidMaskBuffer() {}  // the extension masks live on the GPU
};

class FluidSolver
{
public:
    FluidSolver(FluidSolverMemoryPool mem_pool);
    ~FluidSolver();

    void stepSemiLagrangian(FluidDomain& fluid_domain, MyFloat dt);
    void stepPIC(FluidDomain& fluid_domain, MyFloat dt);
    void stepFLIP(FluidDomain& fluid_domain, MyFloat dt);
    void stepPICFLIP(FluidDomain& fluid_domain, MyFloat dt);

private:
    bool validate(const FluidDomain& fluid_domain);
    void step(FluidDomain& fluid_domain, int method, MyFloat dt);

    FluidSolverMemoryPool _mem_pool;
    int _cg_max_iterations;  // the reference sets 100 (src/FluidSolver.cpp:81)
    double _cg_tolerance;    // Eigen's default: machine epsilon of MyFloat
};

#endif
