"""Console report of the solver construction (the reference's moduls/messages.py).

The report texts are kept identical to the reference's so that logs of a run
read the same; every printed line is also appended to ``msg.log``.

This module restates the reference's GPLv3-licensed Python layer
(hightower8083/chimera) statement by statement to keep its API as a
drop-in; it is a derivative of that code and is distributed under the GNU
General Public License, version 3 or later, as the reference is.
"""
from __future__ import annotations

_TEXTS = {
    "sol/bounds": "Constructing solver with cylindric boundaries:\n"
                  "** left={0:.3g}, right={1:.3g}, radius={2:.3g}",
    "sol/resols": "Spatial and temporal resolutions:\n"
                  "** dx={0:.3g}, dr={1:.3g}, dt={2:.3g}",
    "sol/grdsz": "Grid sizes are:\n** Nx={0:d}, Nr={1:d}, Mo={2:d}",
    "sol/actv": "Solver is active from t={:g} to t={:g}",
    "sol/rcut": "Rgrid is cut after {:.5g} (Nr is reduced to {:d})",
    "sol/shift": "Spectral domain is shifted",
    "sol/echo_intro": "Echo suppression is actived (expert feature)\n"
                      "** To change, set 'AntiEchoStrength' in solvers 'Features',\n"
                      "** or add 'NoAntiEcho' to solvers 'Features' to disactivate",
    "sol/spcchrg": "Charge density will be considered",
    "sol/stillspcs": "\"Still\" species will be treated as background",
    "sol/pois": "Poisson correction will not be performed",
}


class ChimeraMessages:
    """Prints the construction report and keeps it in ``log``."""

    def __init__(self, quiet: bool = False):
        self.msg = dict(_TEXTS)
        self.log: list[str] = []
        self.quiet = quiet

    def print_(self, kw, args=None):
        text = self.msg[kw] if args is None else self.msg[kw].format(*args)
        if not self.quiet:
            print(text)
        self.log.append(text)


msg = ChimeraMessages()
