"""Host-side Python for tdbem-gb300: input format, mesh generators and the
ctypes binding of the C-ABI library (libtdbem.so).  The compute path is the
CUDA library; nothing here computes G/H levels or marches on the CPU."""
from .inputfile import Model, parse, read, dumps, write  # noqa: F401
