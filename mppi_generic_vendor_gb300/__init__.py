"""GB300-native MPPI engine with MPPI-Generic's plugin / controller interface.

The compute path is libmppi_gb.so (hand-written sm_103a CUDA behind the C ABI in include/mppi_gb.h); this package is
the host-side mirror of the reference's interface.  Build the library with ``python -m mppi_generic_vendor_gb300.build``.
"""
from . import _abi
from ._abi import MPPIError
from . import nn_io
from .controller import (BatchedMPPIController, BicycleDynamics, ColoredMPPIController, TubeMPPIController, BicycleSlipDynamics, BicycleSlipMLPDynamics,
                         RobustMPPIController,
                         CartpoleDynamics, DDPFeedback, DDPFeedbackState, DDPParams,
                         CartpoleSwingupCost, ColoredNoiseDistribution, CostmapCost, DoubleIntegratorDynamics,
                         DoubleIntegratorObstacleCost, GaussianDistribution, VanillaMPPIController,
                         select_top_samples)

__all__ = ["MPPIError", "BatchedMPPIController", "VanillaMPPIController", "ColoredMPPIController", "TubeMPPIController", "CartpoleDynamics", "CartpoleSwingupCost",
           "DoubleIntegratorDynamics", "DoubleIntegratorObstacleCost", "BicycleDynamics", "BicycleSlipDynamics",
           "BicycleSlipMLPDynamics",
           "CostmapCost", "GaussianDistribution", "ColoredNoiseDistribution", "select_top_samples", "_abi", "nn_io",
           "DDPFeedback", "DDPFeedbackState", "DDPParams", "RobustMPPIController"]
