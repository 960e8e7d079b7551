from . import gauge
from . import fermion
