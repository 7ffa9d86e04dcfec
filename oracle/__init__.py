"""Oracle: CPU restatement of del-msh-cpu's LBVH build and BVH ray cast.

TEST INFRASTRUCTURE ONLY — what the CUDA path's results are tested against,
and the timed CPU baseline.  The product never imports this package.
"""
