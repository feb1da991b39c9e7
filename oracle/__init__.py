"""Oracle: CPU restatements of the reference's DistMesh path.

TEST INFRASTRUCTURE ONLY.  Nothing under seismicmesh_gb300/ imports this
package; only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use
it, as the checker / the timed reference arm.
"""
