"""CPU oracles of the Voxel ReSTIR render path (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the
checker; the product (smallproject_gb300, libvxr.so) never imports or links it.
"""
