"""Output and checkpoint utilities (utils/dump_vtk.py of the reference, and
engine snapshots)."""
