"""Photon history (excalibur/photon/photon_history.py:19-44)."""
import numpy as np


class PhotonHistory:
    def __init__(self):
        self.states = []

    def append(self, state):
        self.states.append(np.array(state, copy=True))

    def save_to_hdf5(self, filename):
        """The rows as one NaN-padded dataset "states" (photon_history.py:27-44); needs h5py."""
        try:
            import h5py
        except ImportError as e:
            raise RuntimeError("h5py is not available; cannot save PhotonHistory to HDF5.") from e
        with h5py.File(filename, "w") as f:
            f.create_dataset("states", data=self.as_array() if self.states else np.array([]))

    def as_array(self):
        """History padded with NaN to a [n_records, max_cols] array (runner layout)."""
        if not self.states:
            return np.zeros((0, 0))
        w = max(len(s) for s in self.states)
        out = np.full((len(self.states), w), np.nan)
        for i, s in enumerate(self.states):
            out[i, :len(s)] = s
        return out
