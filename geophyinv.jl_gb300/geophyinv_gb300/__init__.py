"""GB300 engine for GeoPhyInv's FDTD hot path.

The CUDA engine (libgpi_fdtd.so, C ABI in include/gpi_fdtd.h) runs the
staggered-grid acoustic/elastic time loop, CPML, sources, receivers and the
adjoint-state gradient; this package is the Python host mirror of the
reference's Julia API (SeisForwExpt, update!, gradient!, lossvalue).
"""
from .fdtd import (AGeomss, AcousticMedium, BornMap, ElasticMedium, FdtdAcoustic, FdtdAcousticBorn,  # noqa
                   FdtdElastic, Fields, L2DistLoss, Recs, SeisForwExpt, Srcs, get_modelvector, gradient,
                   lossvalue, set_born_perturbation, update, update_batch)
from . import fwi  # noqa
from .rrule import NoTangent, misfit, rrule  # noqa
from .setup import Grid, findfreq_peak, ormsby, ricker  # noqa

__all__ = ["AGeomss", "AcousticMedium", "BornMap", "ElasticMedium", "FdtdAcoustic", "FdtdAcousticBorn",
           "FdtdElastic", "Fields", "Grid", "set_born_perturbation",
           "L2DistLoss", "NoTangent", "fwi", "Recs", "SeisForwExpt", "Srcs", "findfreq_peak", "get_modelvector",
           "gradient", "lossvalue", "misfit", "ormsby", "ricker", "rrule", "update", "update_batch"]
