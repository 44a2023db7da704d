"""FFEA trajectory and RNG-checkpoint files for GPU runs.

The formats are FFEA's own, so that its tools read GPU runs and a GPU run
restarts the way ``World::init`` restarts an FFEA run:

- trajectory (``.ftj``): header of ``World::init`` (src/World.cpp:526-548),
  then per frame, for every blob, ``Blob %d, Conformation %d, step %d``, the
  blob state and one line of 10 ``%e`` values per node: position (m),
  velocity (m/s), potential, force (N) for the mass solvers, position and
  zeros for CG_nomass (``Blob::write_nodes_to_file``, src/Blob.cpp:1143-1178);
  then ``*``, the conformation changes and ``*``
  (``World::print_trajectory_and_measurement_files``, src/World.cpp:4125-4180);
- checkpoint (``.fcp``): ``RNGStreams dedicated to the thermal stress: %d``
  and one line of six ``%lu`` words per stream, rewritten in place
  (``World::print_checkpoints``, src/World.cpp:4233-4280), read back as in
  src/World.cpp:330-385.

A GPU handle has one RNG stream per blob (``RNG_PER_BLOB``) or one shared
stream (``RNG_SHARED``, FFEA's single-thread draw order); the checkpoint
lists the handle's streams in blob order (once for a shared stream).

Frames: FFEA prints frame s after the forces of step s and before its
position update, that is the positions and velocities at the start of step
s, and the RNG checkpoint before the draws of step s.  ``Recorder.run``
writes both after s completed GPU steps, which is the same state.  The
force column of the mass solvers holds the last completed solve (step
s - 1); FFEA prints the solve of step s there.
"""
from __future__ import annotations

import os
from typing import Sequence

import numpy as np

from . import params as P

MESO_FORCE = 2.4364705882352941e-11  # include/dimensions.h:37 (energy / length)


# ---------------------------------------------------------------- trajectory
def write_header(fh, nodes_per_blob: Sequence[int]) -> None:
    """World::init's trajectory header, one conformation per blob."""
    fh.write("FFEA_trajectory_file\n\nInitialisation:\nNumber of Blobs %d\nNumber of Conformations" %
             len(nodes_per_blob))
    for _ in nodes_per_blob:
        fh.write(" %d" % 1)
    fh.write("\n")
    for i, n in enumerate(nodes_per_blob):
        fh.write("Blob %d:\t" % i)
        fh.write("Conformation %d Nodes %d\t" % (0, n))
        fh.write("\n")
    fh.write("\n")
    fh.write("*\n")


def _node_lines(pos, vel, force, solver: int) -> str:
    """Blob::write_nodes_to_file's node lines (meso units in, SI out)."""
    n = len(pos)
    cols = np.zeros((n, 10))
    cols[:, 0:3] = pos * P.MESO_LENGTH
    if solver != P.SOLVER_NOMASS:
        cols[:, 3:6] = vel * P.MESO_VELOCITY
        cols[:, 7:10] = force * MESO_FORCE
    # "%e" formats as C's printf does (6 digits after the point, exponent of
    # at least two digits)
    return "".join("%e %e %e %e %e %e %e %e %e %e\n" % tuple(r) for r in cols.tolist())


def write_frame(fh, step: int, blobs: Sequence[tuple], solvers: Sequence[int]) -> None:
    """One frame: blobs = [(pos, vel, force), ...] in meso units."""
    for i, ((pos, vel, force), solver) in enumerate(zip(blobs, solvers)):
        fh.write("Blob %d, Conformation %d, step %d\n" % (i, 0, step))
        fh.write("DYNAMIC\n")
        fh.write(_node_lines(pos, vel, force, solver))
    fh.write("*\n")
    fh.write("Conformation Changes:\n")
    for i in range(len(blobs)):
        fh.write("Blob %d: Conformation %d -> Conformation %d\n" % (i, 0, 0))
    fh.write("*\n")


def read_last_frame(path: str, nodes_per_blob: Sequence[int]):
    """The last completely written frame (the restart read of World::init,
    src/World.cpp:655-760, and Blob::read_nodes_from_file, src/Blob.cpp:
    1268-1310): (step, [(pos, vel), ...]) in meso units."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    # frames are delimited by "*" lines: node data, then conformation changes
    stars = [i for i, ln in enumerate(lines) if ln == "*"]
    nb = len(nodes_per_blob)
    for k in range(len(stars) - 2, 0, -1):
        # a complete frame ends at stars[k + 1] with its conformation block
        start, end = stars[k - 1] + 1, stars[k]
        body = lines[start:end]
        if not body or not body[0].startswith("Blob 0, Conformation"):
            continue
        if lines[end + 1] != "Conformation Changes:" or stars[k + 1] != end + 2 + nb:
            continue
        out, at, step = [], 0, None
        for b, n in enumerate(nodes_per_blob):
            head = body[at].split()
            if head[0] != "Blob" or int(head[1].rstrip(",")) != b:
                raise ValueError(f"{path}: expected blob {b}, found {body[at]!r}")
            step = int(head[-1])
            vals = np.array([[float(x) for x in ln.split()] for ln in body[at + 2:at + 2 + n]])
            if vals.shape != (n, 10):
                raise ValueError(f"{path}: blob {b}: expected {n} node lines of 10 values")
            out.append((vals[:, 0:3] / P.MESO_LENGTH, vals[:, 3:6] / P.MESO_VELOCITY))
            at += 2 + n
        return step, out
    raise ValueError(f"{path}: no completely written frame")


# ---------------------------------------------------------------- checkpoint
def write_checkpoint(path: str, states: Sequence[Sequence[int]]) -> None:
    """World::print_checkpoints: the thermal-stress streams' states."""
    with open(path, "w") as fh:
        fh.write("RNGStreams dedicated to the thermal stress: %d\n" % len(states))
        for st in states:
            fh.write("%d %d %d %d %d %d\n" % tuple(int(x) for x in st))


def read_checkpoint(path: str) -> list:
    """The stream states of a checkpoint, as World::init reads them."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    n = int(lines[0].split(" ")[-1])
    out = []
    for i in range(1, n + 1):
        words = lines[i].split(" ")
        if len(words) != 6:
            raise ValueError(f"{path}: line {i + 1}: expected 6 integers")
        out.append(np.array([int(w) for w in words], dtype=np.uint64))
    return out


# ---------------------------------------------------------------- runs
def stream_states(world) -> list:
    """The handle's RNG streams in blob order (a shared stream once)."""
    states = [world.blob(i).rng_state() for i in range(world.num_blobs)]
    if getattr(world, "rng_mode", None) == 1:  # RNG_SHARED
        return states[:1]
    return states


class Recorder:
    """World::run's output side for a GPU World: every `check` steps the RNG
    checkpoint (rewritten) and a trajectory frame, as FFEA writes them
    (src/World.cpp:2020-2043).  `restart=True` continues an existing pair of
    files: positions and velocities from the last complete frame, RNG states
    from the checkpoint (src/World.cpp:330-385, 655-760), and appends."""

    def __init__(self, world, trajectory: str, checkpoint: str, solvers: Sequence[int], check: int = 1,
                 restart: bool = False):
        if check < 1:
            raise ValueError("check must be >= 1")
        self.world, self.check, self.solvers = world, int(check), list(solvers)
        self.trajectory, self.checkpoint = trajectory, checkpoint
        self.nodes = [world.blob(i).n for i in range(world.num_blobs)]
        self.step = 0
        self._written = -1  # step of the last frame written
        if restart:
            self.step, frame = read_last_frame(trajectory, self.nodes)
            for i, (pos, vel) in enumerate(frame):
                world.blob(i).set_nodes(pos, vel)
            states = read_checkpoint(checkpoint)
            shared = len(states) == 1 and world.num_blobs > 1
            for i in range(world.num_blobs):
                world.blob(i).set_rng_state(states[0 if shared else i])
            # the restart point is written again by the next frame (FFEA
            # truncates the file to the frame it restarts from)
            self._truncate_after_frame(self.step)
        else:
            with open(trajectory, "w") as fh:
                write_header(fh, self.nodes)

    def _truncate_after_frame(self, step: int) -> None:
        with open(self.trajectory) as fh:
            text = fh.read()
        mark = "Blob 0, Conformation 0, step %d\n" % step
        at = text.rfind(mark)
        if at < 0:
            raise ValueError(f"{self.trajectory}: no frame for step {step}")
        with open(self.trajectory, "w") as fh:
            fh.write(text[:at])

    def _frame(self) -> None:
        blobs = [self.world.blob(i).get_nodes() for i in range(self.world.num_blobs)]
        with open(self.trajectory, "a") as fh:
            write_frame(fh, self.step, blobs, self.solvers)

    def _output(self) -> None:
        """Checkpoint and frame of the current state, once per step index."""
        if self.step % self.check == 0 and self.step != self._written:
            write_checkpoint(self.checkpoint, stream_states(self.world))
            self._frame()
            self._written = self.step

    def run(self, num_steps: int) -> None:
        """num_steps steps; at every step s with s % check == 0 the checkpoint
        and the frame of the state before step s are written first."""
        end = self.step + int(num_steps)
        while self.step < end:
            self._output()
            n = min(self.check - self.step % self.check, end - self.step)
            self.world.run(n)
            self.step += n
        self._output()


def restart_files_exist(trajectory: str, checkpoint: str) -> bool:
    return os.path.exists(trajectory) and os.path.exists(checkpoint)
