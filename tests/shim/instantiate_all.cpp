// Instantiates every member of the shim's class templates for each stiffness kind, so that a
// member no other program calls still has to compile (tests/test_shim.py compiles it, no GPU).
#include "alamo_elastic.H"

template class Operator::Elastic<Model::Solid::Linear::Isotropic>;
template class Operator::Elastic<Model::Solid::Linear::Cubic>;
template class Operator::Elastic<Model::Solid::Linear::Laplacian>;
template class Solver::Nonlocal::Newton<Model::Solid::Linear::Isotropic>;
template class Solver::Nonlocal::Newton<Model::Solid::Linear::Cubic>;
template class Operator::Elastic<Model::Solid::Elastic::NeoHookean>;
template class Solver::Nonlocal::Newton<Model::Solid::Elastic::NeoHookean>;

int main() { return 0; }
