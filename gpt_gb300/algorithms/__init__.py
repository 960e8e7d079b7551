from . import inverter
