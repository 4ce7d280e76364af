"""HDF5 export of simulation results in the reference's layout.

The reference saves a run as (trajectory_simulator.py:160-254, beamline.py:78-90,
distributions.py:78-142, apertures.py:56-78, electrostatic_lens.py:145-166,
molecule.py:97-106,169-185):

    <run>/counter                    attrs: label -> count
    <run>/beamline/<element name>    attrs: class, then the element's fields
    <run>/velocity_distribution      attrs: class, then the fields
    <run>/position_distribution      attrs: class, then the fields
    <run>/trajectories/molecule_<i>  datasets x, v, a (n, 3), t (n,); attrs aperture_hit, alive

The classes of this package write the same layout through the functions here.
h5py is imported only when a file is written (it is optional in the reference
too).
"""
from __future__ import annotations

from dataclasses import fields, is_dataclass


def _h5py():
    import h5py

    return h5py


def field_items(obj) -> list:
    """(name, value) of the fields the reference's ``vars(self)`` would list: the
    dataclass fields and the attributes set in ``__post_init__``."""
    return list(vars(obj).items())


def save_element(element, filepath, parent_group_path: str, skip=()) -> None:
    """BeamlineElement.save_to_hdf (apertures.py:56-78); Honeycomb skips its
    patches (meshes.py:172-175)."""
    h5py = _h5py()
    with h5py.File(filepath, "a") as f:
        try:
            group_path = parent_group_path + "/" + element.name
            f.create_group(group_path)
            f[group_path].attrs["class"] = type(element).__name__
            for key, value in field_items(element):
                if key in skip:
                    continue
                f[group_path].attrs[key] = value
        except ValueError:
            print("Can't save beamline element. Group already exists!")


def save_lens(lens, filepath, parent_group_path: str) -> None:
    """ElectrostaticLens.save_to_hdf (electrostatic_lens.py:145-166): the force
    table is not saved, the Stark state and falsy fields as their repr."""
    h5py = _h5py()
    with h5py.File(filepath, "a") as f:
        group_path = parent_group_path + "/" + lens.name
        f.create_group(group_path)
        f[group_path].attrs["class"] = type(lens).__name__
        for key, value in field_items(lens):
            if (key == "dt" and value is None) or (key == "scheme" and value == "reference"):
                continue  # this package's extension fields, at the reference's behaviour
            if key not in ("state", "a_interp") and value:
                f[group_path].attrs[key] = value
            elif key == "a_interp":
                pass
            else:
                f[group_path].attrs[key] = value.__repr__()


def save_beamline(beamline, filepath, run_name: str) -> None:
    """Beamline.save_to_hdf (beamline.py:78-90)."""
    h5py = _h5py()
    with h5py.File(filepath, "a") as f:
        group_path = run_name + "/beamline/"
        f.create_group(group_path)
        for element in beamline.elements:
            element.save_to_hdf(filepath, group_path)


def save_distribution(dist, filepath, run_name: str, group: str, what: str) -> None:
    """CeNTREXVelocityDistribution / *PositionDistribution.save_to_hdf (distributions.py:78-142)."""
    h5py = _h5py()
    with h5py.File(filepath, "a") as f:
        try:
            group_path = run_name + "/" + group
            f.create_group(group_path)
            f[group_path].attrs["class"] = type(dist).__name__
            for key, value in field_items(dist):
                f[group_path].attrs[key] = value
        except ValueError:
            raise ValueError(f"Can't save {what} distribution. Group already exists!")


def save_counter(counter, filepath, run_name: str) -> None:
    """Counter.save_to_hdf (trajectory_simulator.py:160-176)."""
    h5py = _h5py()
    with h5py.File(filepath, "a") as f:
        try:
            group_path = run_name + "/counter"
            f.create_group(group_path)
            for key, value in counter.counter_dict.items():
                f[group_path].attrs[key] = value
        except ValueError:
            raise ValueError("Can't save counter. Group already exists!")


def save_trajectory(traj, file, run_name: str, group_name: str) -> None:
    """Trajectory.save_to_hdf (molecule.py:169-185)."""
    traj.drop_nans()
    group_path = run_name + "/" + group_name
    file.create_group(group_path)
    file[group_path].create_dataset("x", data=traj.x)
    file[group_path].create_dataset("v", data=traj.v)
    file[group_path].create_dataset("a", data=traj.a)
    file[group_path].create_dataset("t", data=traj.t)


def save_molecule(molecule, file, run_name: str, group_name: str) -> None:
    """Molecule.save_to_hdf (molecule.py:97-106)."""
    molecule.trajectory.save_to_hdf(file, run_name, group_name)
    file[run_name + "/" + group_name].attrs["aperture_hit"] = molecule.aperture_hit
    file[run_name + "/" + group_name].attrs["alive"] = molecule.alive


def save_result(result, filepath, run_name: str) -> None:
    """SimulationResult.save_to_hdf (trajectory_simulator.py:218-244): the run
    group (asking before overwriting an existing one), the counter, beamline and
    distributions, then the molecules."""
    h5py = _h5py()
    with h5py.File(filepath, "a") as f:
        try:
            f.create_group(run_name)
        except ValueError:
            val = input("Run name already exists. Overwrite? y/n")
            if val == "y":
                del f[run_name]
                f.create_group(run_name)
            else:
                return
    names = [fl.name for fl in fields(result)] if is_dataclass(result) else list(vars(result))
    for name in names:
        if name in ("molecules", "replay"):
            continue
        getattr(result, name).save_to_hdf(filepath, run_name)
    save_molecules(result, filepath, run_name)


def save_molecules(result, filepath, run_name: str) -> None:
    """SimulationResult.save_molecules_to_hdf (trajectory_simulator.py:246-254)."""
    h5py = _h5py()
    print("Saving trajectories...")
    with h5py.File(filepath, "a") as f:
        for i, molecule in enumerate(result.molecules):
            molecule.save_to_hdf(f, run_name, f"trajectories/molecule_{i}")
