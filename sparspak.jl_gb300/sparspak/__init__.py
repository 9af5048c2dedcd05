"""GB300-native numeric engine behind the Sparspak.jl LU SparseSolver flow.

Module map (reference module -> here):
  SpkProblem          -> sparspak.problem   (Problem, inaij_, inbi_, insparse_, outsparse, ...)
  SpkGraph/SpkOrdering/SpkETree -> sparspak.graph (Graph, Ordering, ETree, mmd_, nd_grid)
  SpkSparseBase/SpkSparseSolver -> sparspak.sparse_solver (SparseSolver, findorder_, ..., solve_)
  SparseCSCInterface  -> sparspak.csc       (sparspaklu, sparspaklu_, ldiv_, ldiv)
Julia's mutating ``f!`` is spelled ``f_``.  Numeric phases run in
libspk_gpu.so (include/spk_gpu.h); there is no CPU fallback.
"""
from . import gallery, graph, problem, sparse_solver
from ._build import build
from .csc import ldiv, ldiv_, sparspaklu, sparspaklu_
from .device import DeviceTimeoutError, ErrorException, NumericEngine, SingularException
from .graph import (ETree, Graph, Ordering, isstructuresymmetric, makestructuresymmetric, mmd_, nd_graph, nd_grid,
                    nd_grid_batched)
from .problem import (Grid, Problem, computeresidual, inaij_, inbi_, infullrhs_, insparse_, makegridproblem,
                      makerhs_, outsparse, zerorhs_)
from .sparse_solver import (SparseSolver, factor_, findorder_, findorderperm_, gradient_, inmatrix_, refine_, solve_,
                            symbolicfactor_, transposetriangularsolve_, triangularsolve_)

__all__ = [
    "build", "gallery", "graph", "problem", "sparse_solver",
    "ldiv", "ldiv_", "sparspaklu", "sparspaklu_",
    "DeviceTimeoutError", "ErrorException", "NumericEngine", "SingularException",
    "ETree", "Graph", "Ordering", "isstructuresymmetric", "makestructuresymmetric", "mmd_", "nd_graph", "nd_grid",
    "nd_grid_batched",
    "Grid", "Problem", "computeresidual", "inaij_", "inbi_", "infullrhs_", "insparse_", "makegridproblem",
    "makerhs_", "outsparse", "zerorhs_",
    "SparseSolver", "factor_", "findorder_", "findorderperm_", "gradient_", "inmatrix_", "refine_", "solve_",
    "symbolicfactor_", "transposetriangularsolve_", "triangularsolve_",
]
