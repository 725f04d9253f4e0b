"""parla_gb300: the randomized-linear-algebra hot path of PARLA on NVIDIA GB300.

Same names and call signatures as the reference package (``parla/__init__.py``):
sketch generators (SkOpGA, SkOpSJ, SkOpTC), RS1, RF1, QB1, QB2, QB3, SVD1, EVD1,
EVD2, SPO, SSO1, SPU1, SPS1, SPS2 and the interpolative decompositions (qrcp_osid,
ROCS1, OSID1, OSID2, TSID1, CUR1).  Products, factorizations and LSQR run in the CUDA
kernels of ``librla_gb300.so`` (C ABI in ``include/rla_gb300.h``).
"""
__version__ = "0.1.0"

from .utils.sketching import (gaussian_operator, sjlt_operator, srct_operator, generate_srct,
                              DeviceOperator, DenseOperator, GaussianOperator, GridGaussianOperator, SJLTOperator,
                              SRCTOperator)
from .comps.sketchers.oblivious import SketchOpGen, SkOpGA, SkOpSJ, SkOpTC
from .comps.sketchers.aware import RowSketcher, RS1
from .comps.rangefinders import RangeFinder, RF1
from .comps.qb import QBDecomposer, QB1, QB2, QB3
from .comps.determiter.logging import SketchAndPrecondLog
from .comps.determiter.saddle import PrecondSaddleSolver, PcSS1, PcSS2
from .comps.determiter.pcg import pcg
from .comps.determiter.lsqr import lsqr, PrecondOperator
from .drivers.least_squares import OverLstsqSolver, UnderLstsqSolver, SPO, SSO1, SPU1, dim_checks
from .drivers.saddlesys import SaddleSolver, SPS1, SPS2
from .drivers.batched import BatchedSPO
from .drivers.svd import SVDecomposer, SVD1
from .drivers.evd import EVDecomposer, EVD1, EVD2
from .comps.interpolative import qrcp_osid, RowOrColSelection, ROCS1, rocs1
from .drivers.interpolative import (OneSidedID, OSID1, OSID2, osid1, osid2, TwoSidedID, TSID1, tsid1,
                                    CURDecomposition, CUR1, cur1)
from .utils.linalg_wrappers import orth, cholqr
from .autotune import Tuner
