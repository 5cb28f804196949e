// sf_stubs.cpp -- launchers not implemented yet
#include "sf_internal.h"
#include "sf_launch.h"
namespace sf {
int launch_cont_diagonal(const sf_op *, int, void *, cudaStream_t)
{ set_error("diagonal not built yet"); return SF_ERR_UNSUPPORTED; }
}
extern "C" void sf_solve_opts_default(sf_solve_opts *o)
{
  o->mode = SF_SOLVE_FP64; o->precond = SF_PRECOND_NONE; o->cheb_degree = 5; o->cheb_range = 15.0;
  o->eig_iterations = 12; o->rtol = 1e-10; o->max_iter = 10000; o->inner_rtol = 1e-3; o->project_constant = 0;
}
extern "C" int sf_cg_solve(sf_op *, const double *, double *, const sf_solve_opts *, sf_solve_stats *, void *)
{ sf::set_error("solver not built yet"); return SF_ERR_UNSUPPORTED; }
