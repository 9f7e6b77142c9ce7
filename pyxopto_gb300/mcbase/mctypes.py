"""Data type descriptors (xopto/mcbase/mctypes.py:766-900).  The GB300
kernels compute in single precision with 64-bit accumulators and a 64-bit
packet counter; McDataTypesSingle is the only accepted set."""
import numpy as np


class McDataTypesSingle:
    mc_accu_k = 0x7FFFFF
    mc_cnt_max = 2 ** 64 - 1
    np_float = 'float32'
    np_accu = 'uint64'
    np_cnt = 'uint64'
    np_int = 'int32'
    eps = float(np.finfo(np.float32).eps)


McDataTypes = McDataTypesSingle
McDataTypesSingleCnt64 = McDataTypesSingle


def check(types):
    if types not in (None, McDataTypesSingle) and not (
            isinstance(types, type) and issubclass(types, McDataTypesSingle)):
        name = getattr(types, '__name__', str(types))
        if 'Double' in name:
            raise ValueError('Double precision is not supported by the GB300 kernels.')
    return McDataTypesSingle
