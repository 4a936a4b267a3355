"""Owned result arrays of one MONKI product and their NetCDF storage.

Mirrors the reference's ``SimulationResult`` (python/monki/output/__init__.py:10-74):
variable values, dimension names and attributes, copied out of the file on load, and an
exclusive-create save that never replaces an existing product. The reference writes
NetCDF-4 through ``netCDF4``; where that package is absent the product is written as
NetCDF-3 (64-bit offset) through ``scipy.io``, with identical names, dimensions, types
and attributes.
"""

from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

try:  # pragma: no cover - depends on the host image
    import netCDF4 as _netcdf4
except ImportError:  # pragma: no cover
    _netcdf4 = None


@dataclass(frozen=True)
class SimulationResult:
    """Data, dimension names and units of one MONKI NetCDF product."""

    path: Path | None
    values: dict[str, np.ndarray]
    dimensions: dict[str, tuple[str, ...]]
    attributes: dict[str, dict]

    @classmethod
    def load(cls, path: str | Path) -> "SimulationResult":
        """Copy every variable out of the file; masked (missing) values are rejected."""

        path = Path(path).resolve()
        values, dimensions, attributes = {}, {}, {}

        if _netcdf4 is not None:
            with _netcdf4.Dataset(path) as dataset:
                for name, variable in dataset.variables.items():
                    data = variable[:]

                    if np.ma.isMaskedArray(data) and np.any(np.ma.getmaskarray(data)):
                        raise ValueError(f"{name}: masked/missing data in {path}")

                    values[name] = np.array(data, copy=True)
                    dimensions[name] = tuple(variable.dimensions)
                    attributes[name] = {key: variable.getncattr(key) for key in variable.ncattrs()}

            return cls(path, values, dimensions, attributes)

        from scipy.io import netcdf_file

        with netcdf_file(path, "r", mmap=False) as dataset:
            for name, variable in dataset.variables.items():
                values[name] = np.array(variable.data, copy=True)
                dimensions[name] = tuple(variable.dimensions)
                attributes[name] = {
                    key: (value.decode() if isinstance(value, bytes) else value)
                    for key, value in variable._attributes.items()
                }

        return cls(path, values, dimensions, attributes)

    def save(self) -> None:
        """Write the product, refusing to replace an existing file."""

        if self.path is None:
            raise ValueError("SimulationResult has no output path")

        path = Path(self.path)
        path.parent.mkdir(parents=True, exist_ok=True)
        sizes: dict[str, int] = {}

        for name, value in self.values.items():
            for dimension, size in zip(self.dimensions[name], value.shape, strict=True):
                if dimension in sizes and sizes[dimension] != size:
                    raise ValueError(f"Inconsistent dimension {dimension}")

                sizes[dimension] = size

        if _netcdf4 is not None:
            with _netcdf4.Dataset(path, "w", clobber=False) as dataset:
                for name, size in sizes.items():
                    dataset.createDimension(name, size)

                for name, value in self.values.items():
                    variable = dataset.createVariable(name, value.dtype, self.dimensions[name])
                    variable.setncatts(self.attributes.get(name, {}))
                    variable[:] = value

            return

        from scipy.io import netcdf_file

        # Exclusive creation protects an existing product even against a racing writer.
        with open(path, "xb") as stream, netcdf_file(stream, "w", version=2) as dataset:
            for name, size in sizes.items():
                dataset.createDimension(name, size)

            for name, value in self.values.items():
                data = np.asarray(value)

                if data.dtype == np.int64:
                    data = data.astype(np.int32)

                variable = dataset.createVariable(name, data.dtype, self.dimensions[name])

                for key, attribute in self.attributes.get(name, {}).items():
                    setattr(variable, key, attribute)

                variable[...] = data

    @property
    def radiance(self) -> np.ndarray:
        return self.values["radiance"]

    @property
    def standard_error(self) -> np.ndarray:
        return self.values["std_radiance"]
