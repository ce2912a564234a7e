"""Helpers of the reference's backend/utils.py: boundary planes, the
empirical marching-time model, and mesh simplification via meshlabserver."""
from __future__ import annotations

import os
import subprocess
import tempfile

import torch


def get_boundary(boundary_type="cube", **kwargs):
    """The 6 half-spaces w.x + b < 0 of an axis-aligned cube
    (backend/utils.py:5-29): min_vert / max_vert corners."""
    if boundary_type != "cube":
        raise ValueError("No such %s" % boundary_type)
    mx, mn = kwargs["max_vert"], kwargs["min_vert"]
    w = torch.tensor([[1, 0, 0], [0, 1, 0], [0, 0, 1], [-1, 0, 0], [0, -1, 0], [0, 0, -1]], dtype=torch.float32)
    b = torch.tensor([-mx[0], -mx[1], -mx[2], mn[0], mn[1], mn[2]], dtype=torch.float32)
    return w, b


def estimate_am_time(model):
    """The reference's fitted time model t(l, n) = (a n)^(b l + c) n^d l^e f
    (backend/utils.py:76-90), l = depth, n = mean hidden width.  A property
    of the reference's implementation, kept for API compatibility."""
    nodes = model.nodes
    depth = len(nodes) - 2
    width = sum(nodes[1:-1]) / depth
    a, b, c, d, e, f = 1.94452188, 0.13816182, -0.14536181, 0.59338494, -1.20459825, 1.17841059
    return (a * width) ** (b * depth + c) * (width ** d) * (depth ** e) * f


_SIMPLIFY = """<!DOCTYPE FilterScript>
<FilterScript>
 <filter name="Simplification: Quadric Edge Collapse Decimation">
  <Param name="TargetFaceNum" value="100000" type="RichInt"/>
  <Param name="TargetPerc" value="{perc}" type="RichFloat"/>
  <Param name="QualityThr" value="0.5" type="RichFloat"/>
  <Param name="PreserveBoundary" value="false" type="RichBool"/>
  <Param name="BoundaryWeight" value="1" type="RichFloat"/>
  <Param name="PreserveNormal" value="true" type="RichBool"/>
  <Param name="PreserveTopology" value="false" type="RichBool"/>
  <Param name="OptimalPlacement" value="true" type="RichBool"/>
  <Param name="PlanarQuadric" value="true" type="RichBool"/>
  <Param name="PlanarWeight" value="0.001" type="RichFloat"/>
  <Param name="QualityWeight" value="false" type="RichBool"/>
  <Param name="AutoClean" value="true" type="RichBool"/>
  <Param name="Selected" value="false" type="RichBool"/>
 </filter>
 <filter name="Select non Manifold Edges "/>
 <filter name="Delete Selected Faces"/>
 <filter name="Close Holes">
  <Param name="MaxHoleSize" value="100" type="RichInt"/>
  <Param name="Selected" value="false" type="RichBool"/>
  <Param name="NewFaceSelected" value="true" type="RichBool"/>
  <Param name="SelfIntersection" value="true" type="RichBool"/>
 </filter>
</FilterScript>
"""


def simplify(ply_path, save_ply_path=None, target_perc=0.01, meshlabserver_path="meshlabserver"):
    """Quadric decimation through an external meshlabserver
    (backend/utils.py:31-74); returns its exit status."""
    with tempfile.TemporaryDirectory() as d:
        script = os.path.join(d, "script.mlx")
        with open(script, "w") as f:
            f.write(_SIMPLIFY.format(perc=target_perc))
        out = ply_path if save_ply_path is None else save_ply_path
        try:
            return subprocess.call([meshlabserver_path, "-i", ply_path, "-o", out, "-s", script])
        except FileNotFoundError:
            raise RuntimeError("meshlabserver not found: %s" % meshlabserver_path)
