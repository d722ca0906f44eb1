"""Device-resident process tensor for the reference's ``compute_dynamics``.

``DeviceProcessTensor`` subclasses the reference's abstract
``BaseProcessTensor`` (oqupy/process_tensor.py:38-197) and keeps the PT-MPO
tensors and caps of a GPU PT-TEMPO build in device memory.  The accessors
of the abstract interface copy one tensor to the host on demand, in the
reference's conventions:

* ``get_mpo_tensor(step, transformed=True)``: rank-4 ``[past bond, future
  bond, in, out]`` with the delta between the system legs made explicit and
  ``transform_in`` / ``transform_out`` applied (as
  ``SimpleProcessTensor.get_mpo_tensor``, process_tensor.py:326-356);
* ``get_cap_tensor(step)``: the cap vector computed on the device when the
  build completed (``SimpleProcessTensor.compute_caps``, :380-406), ``None``
  out of range (:358-365);
* ``get_bond_dimensions()``: ``num_steps + 1`` bond dimensions (:367-378).

``compute_dynamics`` (rebound by ``oqupy_gb300.install``) sweeps a
``DeviceProcessTensor`` on the GPU without copying any tensor to the host.
The class is created against the ``BaseProcessTensor`` of the ``oqupy``
package in use (``device_process_tensor_class``), since the reference is the
package's host, not a dependency of the engine.
"""

from typing import Any, Dict, Optional

import numpy as np

_classes: Dict[int, type] = {}


def device_process_tensor_class(base_cls: Any) -> type:
    """``DeviceProcessTensor`` built on the given ``BaseProcessTensor``."""
    key = id(base_cls)
    if key in _classes:
        return _classes[key]

    class DeviceProcessTensor(base_cls):
        """PT-MPO of one GPU PT-TEMPO build (``PtBatch`` entry ``index``),
        kept in device memory."""

        def __init__(self, batch, index: int, hilbert_space_dimension: int,
                     dt: Optional[float] = None, transform_in=None, transform_out=None,
                     name: Optional[str] = None, description: Optional[str] = None):
            super().__init__(hilbert_space_dimension, dt, transform_in, transform_out,
                             name, description)
            self._batch = batch
            self._index = int(index)
            self._len = int(batch.meta[self._index]["num_steps"])

        def __len__(self) -> int:
            return self._len

        @property
        def device(self):
            """``(PtBatch, index)`` of the device tensors."""
            return self._batch, self._index

        def get_initial_tensor(self):
            return None

        def get_mpo_tensor(self, step: int, transformed: Optional[bool] = True) -> np.ndarray:
            if step >= self._len or step < 0:
                raise IndexError("Process tensor index out of bound. ")
            t3 = self._batch.mpo_tensor(self._index, step)
            tensor = np.einsum("lra,ab->lrab", t3, np.eye(t3.shape[2], dtype=t3.dtype))
            if transformed is False:
                return tensor
            if self._transform_in is not None:
                tensor = np.moveaxis(np.dot(np.moveaxis(tensor, -2, -1), self._transform_in.T), -1, -2)
            if self._transform_out is not None:
                tensor = np.dot(tensor, self._transform_out)
            return tensor

        def get_cap_tensor(self, step: int):
            if step > self._len or step < 0:
                return None
            return self._batch.cap(self._index, step)

        def get_bond_dimensions(self) -> np.ndarray:
            return self._batch.bond_dimensions(self._index)

        def compute_caps(self) -> None:
            """The caps are computed on the device when the build completes."""

        def to_host(self, simple_cls):
            """A host copy as ``simple_cls`` (the reference's
            ``SimpleProcessTensor``): rank-3 tensors and caps."""
            pt = simple_cls(self._hs_dim, self._dt, self._transform_in, self._transform_out,
                            self.name, self.description)
            for step in range(self._len):
                pt.set_mpo_tensor(step, self._batch.mpo_tensor(self._index, step))
            pt.compute_caps()
            return pt

    _classes[key] = DeviceProcessTensor
    return DeviceProcessTensor
