"""GB300-native (sm_103a) density-matrix hot path of largeTB.

The product is the C-ABI shared library built from ``largetb_gb300/csrc``
(declared in ``include/largetb.h``); this package builds it in-tree and
exposes it to Python through ctypes (``largetb_gb300.api``).
"""
from .api import (  # noqa: F401
    MLP, Batch, Context, Model, TbError, mlp_features, TbParams, TbReport, load, model_cristobalite, model_quartz, params,
    PREC_FP32, PREC_FP64, KERNEL_AUTOCORR, KERNEL_JACKSON, KERNEL_NONE,
    FP32_AUTO, FP32_STAGED, FP32_PERSISTENT, FP32_PIPELINED, FP32_PIPELINED_STEP, MODE_KPE, MODE_SP2,
)
from .build import build as build_library  # noqa: F401
