"""GB300-native (sm_103a) batched transaction-processing hot path.

The product is the C ABI in include/ltpmg_gb300.h implemented by
libltpmg_gb300.so (hand-written CUDA); this package is its ctypes binding.
"""
from .lib import (Batch, Context, Ingest, LtpError, PinnedArray, Pipe, Server, RULE_ORDERED, RULE_PRIORITY, OP_ADD, OP_READ,  # noqa: F401
                  OP_INSERT, MODE_STREAM, MODE_GRAPH, MODE_PERSISTENT, TPCC_TABLES, Tpcc,
                  gen_ycsb, header_functions, load, opword)
