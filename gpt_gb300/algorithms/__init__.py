from . import inverter, modes
