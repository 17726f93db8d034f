"""GB300-native moving-least-squares point-cloud transfer (DataTransferKit MLS path).

The compute path is ``libdtk_gb300.so`` (hand-written sm_103a CUDA behind the
C ABI of ``include/dtk_gb300.h``); this package is its host-side mirror of
DataTransferKit's operator API.  There is no CPU fallback.
"""
from .operators import (FP64, MIXED, Buhmann, Constant, Linear, MovingLeastSquaresBatch,
                        MovingLeastSquaresOperator, NearestNeighborOperator,
                        MultivariatePolynomialBasis, PointCloudOperator, Quadratic, Wendland, Wu,
                        kernel_launch_count, knn_search, release_cached_memory, set_setup_lanes,
                        svd_pinv)
from ._capi import DTKError, InvalidArgument, Unsupported
from .distributed import DistributedMovingLeastSquaresOperator, DistributedNearestNeighborOperator, fetch

__all__ = ["MovingLeastSquaresOperator", "MovingLeastSquaresBatch", "NearestNeighborOperator", "PointCloudOperator", "MultivariatePolynomialBasis",
           "Constant", "Linear", "Quadratic", "Wendland", "Wu", "Buhmann", "FP64", "MIXED",
           "knn_search", "svd_pinv", "DistributedMovingLeastSquaresOperator",
           "DistributedNearestNeighborOperator", "fetch", "kernel_launch_count", "release_cached_memory", "set_setup_lanes", "DTKError", "InvalidArgument", "Unsupported"]
