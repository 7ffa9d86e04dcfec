"""Oracle: CPU restatement of del-msh-cpu's LBVH build and BVH ray cast.

TEST INFRASTRUCTURE ONLY — the checker for the CUDA path and the timed CPU
baseline.  The product never imports this package.
"""
