"""GB300-native DVS hot path (BVH ray casting, Hapke shading, pixel circuit,
event readout) behind a C-ABI; see include/dvs_gb300.h."""
from ._capi import (EVENT_DTYPE, INTERVAL_DTYPE, STATE_DTYPE, CapacityError, DvsError, OpticalError,  # noqa: F401
                    library_path, load)
from .raycast import (CamRayCaster, DeviceScene, DvsRayCaster, EventSensor, SensorBatch,  # noqa: F401
                      derive_parameters, interval_array, state_array)
