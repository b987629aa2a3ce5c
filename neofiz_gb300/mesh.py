"""Mesh inputs: the flat structure-of-arrays quad mesh and the generators that feed the solver.

``QuadMesh`` mirrors mesh/QuadMesh.java:17-54 (CCW winding checked at construction, :228-237),
``solidCylinder``/``cylinderWall`` mirror :254-356 and the node-set helpers :362-402.
``Outline`` mirrors the lattice mesher mesh/Outline.java: point-in-polygon by crossings
(:136-151), lattice anchored at the origin (:302-309), nodes numbered in first-appearance order
over the row-major cell scan (:317-345, :361-371), and ``assemble`` (:254-287) which meshes
each body separately so that bodies which touch do not share nodes.

Floating-point expressions follow the Java ones term for term, so the coordinates produced
here are bit-identical to the reference's.
"""
from __future__ import annotations

import math
from typing import List, Sequence

import numpy as np


class QuadMesh:
    def __init__(self, r, z, conn, pressureEdges=()):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1)
        pe = np.ascontiguousarray(pressureEdges, dtype=np.int32).reshape(-1)
        if r.shape != z.shape:
            raise ValueError("r and z must have the same length")
        if conn.size % 4 != 0:
            raise ValueError("connectivity must be a multiple of 4")
        if pe.size % 2 != 0:
            raise ValueError("pressure edges must be a multiple of 2")
        self.r, self.z, self.conn, self.pressureEdges = r, z, conn, pe
        self.nodeCount = int(r.size)
        self.elementCount = int(conn.size // 4)
        self._checkOrientation()

    # -- geometry (QuadMesh.java:59-135)
    def signedAreas(self) -> np.ndarray:
        c = self.conn.reshape(-1, 4)
        a = np.zeros(self.elementCount)
        for k in range(4):
            i, j = c[:, k], c[:, (k + 1) % 4]
            a = a + (self.r[i] * self.z[j] - self.r[j] * self.z[i])
        return 0.5 * a

    def signedArea(self, element: int) -> float:
        b = element * 4
        a = 0.0
        for k in range(4):
            i = int(self.conn[b + k]); j = int(self.conn[b + (k + 1) % 4])
            a += float(self.r[i]) * float(self.z[j]) - float(self.r[j]) * float(self.z[i])
        return 0.5 * a

    def _centroids(self, coord: np.ndarray) -> np.ndarray:
        c = self.conn.reshape(-1, 4)
        a = np.zeros(self.elementCount)
        moment = np.zeros(self.elementCount)
        for k in range(4):
            i, j = c[:, k], c[:, (k + 1) % 4]
            cross = self.r[i] * self.z[j] - self.r[j] * self.z[i]
            a = a + cross
            moment = moment + (coord[i] + coord[j]) * cross
        return moment / (3.0 * a)

    def centroidRadii(self) -> np.ndarray:
        return self._centroids(self.r)

    def centroidZs(self) -> np.ndarray:
        return self._centroids(self.z)

    def centroidRadius(self, e: int) -> float:
        return float(self.centroidRadii()[e])

    def centroidZ(self, e: int) -> float:
        return float(self.centroidZs()[e])

    def minimumEdgeLength(self) -> float:
        c = self.conn.reshape(-1, 4)
        best = math.inf
        for k in range(4):
            i, j = c[:, k], c[:, (k + 1) % 4]
            dr = self.r[j] - self.r[i]
            dz = self.z[j] - self.z[i]
            best = min(best, float(np.min(np.sqrt(dr * dr + dz * dz))) if len(dr) else best)
        return best

    def ringVolume(self, element: int) -> float:
        return 2.0 * math.pi * self.centroidRadius(element) * self.signedArea(element)

    def _checkOrientation(self):
        if self.elementCount == 0:
            return
        areas = self.signedAreas()
        bad = np.nonzero(areas <= 0.0)[0]
        if bad.size:
            raise RuntimeError(f"element {int(bad[0])} has non-positive area; node ordering "
                               f"must be counter-clockwise in (r, z)")

    # -- free surface (QuadMesh.java:188-226)
    def surface(self, skip=None):
        """(edges [2S], owner [S], nodes ascending) of the edges owned by one live element."""
        c = self.conn.reshape(-1, 4)
        live = np.ones(self.elementCount, dtype=bool) if skip is None else ~np.asarray(skip, bool)
        a = c
        b = np.roll(c, -1, axis=1)
        lo = np.minimum(a, b).astype(np.int64)
        hi = np.maximum(a, b).astype(np.int64)
        key = (lo << 32) | hi
        lk = key[live].reshape(-1)
        uniq, counts = np.unique(lk, return_counts=True)
        cnt = dict(zip(uniq.tolist(), counts.tolist()))
        edges, owner = [], []
        for e in np.nonzero(live)[0]:
            for k in range(4):
                if cnt[int(key[e, k])] == 1:
                    edges += [int(a[e, k]), int(b[e, k])]
                    owner.append(int(e))
        nodes = np.unique(np.array(edges, dtype=np.int32)) if edges else np.zeros(0, np.int32)
        return (np.array(edges, dtype=np.int32), np.array(owner, dtype=np.int32),
                nodes.astype(np.int32))

    # -- generators
    @staticmethod
    def cylinderWall(innerRadius, outerRadius, height, nr, nz) -> "QuadMesh":
        if outerRadius <= innerRadius:
            raise ValueError("outer radius must exceed inner radius")
        if nr < 1 or nz < 1:
            raise ValueError("need at least one element in each direction")
        nodesR, nodesZ = nr + 1, nz + 1
        r = np.empty(nodesR * nodesZ)
        z = np.empty(nodesR * nodesZ)
        for j in range(nodesZ):
            for i in range(nodesR):
                n = j * nodesR + i
                r[n] = innerRadius + (outerRadius - innerRadius) * i / nr
                z[n] = height * j / nz
        conn = _structuredConn(nr, nz)
        edges = np.empty(nz * 2, dtype=np.int32)
        for j in range(nz):
            edges[2 * j] = j * nodesR
            edges[2 * j + 1] = (j + 1) * nodesR
        return QuadMesh(r, z, conn, edges)

    @staticmethod
    def solidCylinder(radius, height, nr, nz) -> "QuadMesh":
        if radius <= 0.0:
            raise ValueError("radius must be positive")
        if height <= 0.0:
            raise ValueError("height must be positive")
        if nr < 1 or nz < 1:
            raise ValueError("need at least one element in each direction")
        nodesR, nodesZ = nr + 1, nz + 1
        i = np.tile(np.arange(nodesR, dtype=np.float64), nodesZ)
        j = np.repeat(np.arange(nodesZ, dtype=np.float64), nodesR)
        # Java: radius * i / nr, left to right, int promoted to double.
        r = (radius * i) / float(nr)
        z = (height * j) / float(nz)
        return QuadMesh(r, z, _structuredConn(nr, nz), np.zeros(0, np.int32))

    @staticmethod
    def axisNodes(nr, nz):
        return QuadMesh.innerSurfaceNodes(nr, nz)

    @staticmethod
    def nearFaceNodes(nr, nz):
        return list(range(nr + 1))

    @staticmethod
    def farFaceNodes(nr, nz):
        return [nz * (nr + 1) + i for i in range(nr + 1)]

    @staticmethod
    def innerSurfaceNodes(nr, nz):
        return [j * (nr + 1) for j in range(nz + 1)]

    @staticmethod
    def outerSurfaceNodes(nr, nz):
        return [j * (nr + 1) + nr for j in range(nz + 1)]

    @staticmethod
    def axialEndNodes(nr, nz):
        return list(range(nr + 1)) + [nz * (nr + 1) + i for i in range(nr + 1)]


def _structuredConn(nr: int, nz: int) -> np.ndarray:
    nodesR = nr + 1
    j, i = np.meshgrid(np.arange(nz), np.arange(nr), indexing="ij")
    j = j.reshape(-1); i = i.reshape(-1)
    conn = np.stack([j * nodesR + i, j * nodesR + i + 1,
                     (j + 1) * nodesR + i + 1, (j + 1) * nodesR + i], axis=1)
    return conn.reshape(-1).astype(np.int32)


class Outline:
    """A polygon with optional holes, meshed onto a square lattice (mesh/Outline.java)."""

    def __init__(self, ring: Sequence[float], holes: List[Sequence[float]] = None):
        self.ring = [float(v) for v in ring]
        self.holes = [list(h) for h in (holes or [])]

    @staticmethod
    def of(*rz: float) -> "Outline":
        if len(rz) < 6 or len(rz) % 2 != 0:
            raise ValueError(f"a polygon needs at least three (r, z) pairs; got {len(rz)} numbers")
        return Outline(rz)

    @staticmethod
    def rectangle(r0, z0, r1, z1) -> "Outline":
        if r1 <= r0 or z1 <= z0:
            raise ValueError("rectangle needs r1 > r0 and z1 > z0")
        return Outline.of(r0, z0, r1, z0, r1, z1, r0, z1)

    @staticmethod
    def circle(centreR, centreZ, radius, sides) -> "Outline":
        if radius <= 0.0:
            raise ValueError("radius must be positive")
        if sides < 3:
            raise ValueError("need at least three sides")
        rz = []
        for k in range(sides):
            a = 2.0 * math.pi * k / sides
            rz += [centreR + radius * math.cos(a), centreZ + radius * math.sin(a)]
        return Outline(rz)

    def _mapped(self, move) -> "Outline":
        def mv(p):
            out = list(p)
            for i in range(0, len(out), 2):
                out[i], out[i + 1] = move(out[i], out[i + 1])
            return out
        return Outline(mv(self.ring), [mv(h) for h in self.holes])

    def translated(self, dr, dz) -> "Outline":
        return self._mapped(lambda r, z: (r + dr, z + dz))

    def rotated(self, radians, aboutR, aboutZ) -> "Outline":
        c, s = math.cos(radians), math.sin(radians)

        def mv(r, z):
            dr, dz = r - aboutR, z - aboutZ
            return aboutR + c * dr - s * dz, aboutZ + s * dr + c * dz
        return self._mapped(mv)

    def restingOn(self, z) -> "Outline":
        lowest = min(self.ring[1::2])
        return self.translated(0.0, z - lowest)

    def withHole(self, hole: "Outline") -> "Outline":
        return Outline(self.ring, self.holes + [list(hole.ring)] + [list(h) for h in hole.holes])

    @staticmethod
    def _crosses(p, r, z) -> bool:
        inside = False
        n = len(p) // 2
        j = n - 1
        for i in range(n):
            ri, zi = p[2 * i], p[2 * i + 1]
            rj, zj = p[2 * j], p[2 * j + 1]
            if (zi > z) != (zj > z) and r < (rj - ri) * (z - zi) / (zj - zi) + ri:
                inside = not inside
            j = i
        return inside

    def contains(self, r, z) -> bool:
        inside = Outline._crosses(self.ring, r, z)
        for h in self.holes:
            if Outline._crosses(h, r, z):
                inside = not inside
        return inside

    def _containsMany(self, r: np.ndarray, z: np.ndarray) -> np.ndarray:
        def cross(p):
            inside = np.zeros(r.shape, dtype=bool)
            n = len(p) // 2
            j = n - 1
            for i in range(n):
                ri, zi = p[2 * i], p[2 * i + 1]
                rj, zj = p[2 * j], p[2 * j + 1]
                straddle = (zi > z) != (zj > z)
                with np.errstate(divide="ignore", invalid="ignore"):
                    xr = (rj - ri) * (z - zi) / (zj - zi) + ri
                inside ^= straddle & (r < xr)
                j = i
            return inside
        out = cross(self.ring)
        for h in self.holes:
            out ^= cross(h)
        return out

    @staticmethod
    def _shoelace(p) -> float:
        a = 0.0
        n = len(p) // 2
        j = n - 1
        for i in range(n):
            a += p[2 * j] * p[2 * i + 1] - p[2 * i] * p[2 * j + 1]
            j = i
        return 0.5 * a

    def area(self) -> float:
        a = abs(Outline._shoelace(self.ring))
        for h in self.holes:
            a -= abs(Outline._shoelace(h))
        return a

    def bounds(self):
        rs, zs = self.ring[0::2], self.ring[1::2]
        return [min(rs), min(zs), max(rs), max(zs)]

    def centre(self):
        b = self.bounds()
        return [0.5 * (b[0] + b[2]), 0.5 * (b[1] + b[3])]

    def mesh(self, cellSize) -> QuadMesh:
        return Outline.meshOf(cellSize, self)

    @staticmethod
    def meshOf(cellSize, *shapes: "Outline") -> QuadMesh:
        """Outline.mesh(cellSize, shapes...), Outline.java:289-359."""
        if not (cellSize > 0.0):
            raise ValueError(f"cell size must be positive, was {cellSize}")
        if not shapes:
            raise ValueError("nothing to mesh")
        rlo = min(s.bounds()[0] for s in shapes)
        zlo = min(s.bounds()[1] for s in shapes)
        rhi = max(s.bounds()[2] for s in shapes)
        zhi = max(s.bounds()[3] for s in shapes)
        i0 = int(math.floor(rlo / cellSize))
        i1 = int(math.ceil(rhi / cellSize))
        j0 = int(math.floor(zlo / cellSize))
        j1 = int(math.ceil(zhi / cellSize))
        if (i1 - i0) * (j1 - j0) > 20_000_000:
            raise ValueError(f"a cell size of {cellSize} m over this bounding box would need "
                             f"more than twenty million cells; the shape is large or the cell small")
        ni, nj = i1 - i0, j1 - j0
        jj, ii = np.meshgrid(np.arange(j0, j1), np.arange(i0, i1), indexing="ij")
        cr = (ii + 0.5) * cellSize
        cz = (jj + 0.5) * cellSize
        inside = np.zeros(cr.shape, dtype=bool)
        for s in shapes:
            inside |= s._containsMany(cr, cz)
        cells_i = ii[inside]
        cells_j = jj[inside]          # row-major order: j outer, i inner
        if cells_i.size == 0:
            raise ValueError(f"no cell centre fell inside the outline; the shape is smaller "
                             f"than one {cellSize} m cell, or the coordinates are not in metres")
        # Corner lattice coordinates in emission order: (i,j), (i+1,j), (i+1,j+1), (i,j+1).
        ci = np.stack([cells_i, cells_i + 1, cells_i + 1, cells_i], axis=1).reshape(-1)
        cj = np.stack([cells_j, cells_j, cells_j + 1, cells_j + 1], axis=1).reshape(-1)
        key = (ci.astype(np.int64) - (i0 - 1)) * (nj + 3) + (cj.astype(np.int64) - (j0 - 1))
        # First-appearance numbering, as the HashMap walk assigns it.
        uniq, first, inverse = np.unique(key, return_index=True, return_inverse=True)
        order = np.argsort(first, kind="stable")
        rank = np.empty_like(order)
        rank[order] = np.arange(order.size)
        conn = rank[inverse].astype(np.int32)
        node_i = ci[first[order]].astype(np.float64)
        node_j = cj[first[order]].astype(np.float64)
        r = node_i * cellSize
        z = node_j * cellSize
        return QuadMesh(r, z, conn, np.zeros(0, np.int32))

    @staticmethod
    def assemble(cellSize, *shapes: "Outline") -> QuadMesh:
        """Outline.assemble, Outline.java:254-287: bodies meshed separately, nodes offset."""
        if not shapes:
            raise ValueError("nothing to mesh")
        rs, zs, conns = [], [], []
        nodes = 0
        for shape in shapes:
            body = Outline.meshOf(cellSize, shape)
            rs.append(body.r)
            zs.append(body.z)
            conns.append(body.conn + nodes)
            nodes += body.nodeCount
        return QuadMesh(np.concatenate(rs), np.concatenate(zs), np.concatenate(conns),
                        np.zeros(0, np.int32))
