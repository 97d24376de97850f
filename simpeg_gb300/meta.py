"""Meta-simulations over GPU simulations (mirror of ``simpeg.meta``).

``MetaSimulation``, ``SumMetaSimulation`` and ``RepeatedSimulation`` follow
``simpeg/meta/simulation.py:13-520``: every child simulation sees
``mapping * m``; the data are the children's data concatenated (summed for
``SumMetaSimulation``); ``Jvec`` passes ``mapping.deriv(m) @ v`` to each child,
``Jtvec`` sums ``mapping.deriv(m).T @ child.Jtvec``; ``getJtJdiag`` uses the
reference's column-norm form ``sum((diag(sqrt(child diag)) @ deriv)^2)``.

On the GPU the children of a ``MetaSimulation`` / ``SumMetaSimulation`` run
at the same time: each child has its own CUDA stream, driven from its own
host thread (the library's ctypes calls release the GIL), so the solves of
several problems overlap on one device.  ``MultiprocessingMetaSimulation``
(``simpeg/meta/multiprocessing.py``) keeps the reference's name and
``n_processes`` argument for that concurrency: worker processes of their own
would compete for the one GPU instead.
"""

from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.sparse as sp

__all__ = ["MetaSimulation", "SumMetaSimulation", "RepeatedSimulation", "MultiprocessingMetaSimulation",
           "MultiprocessingSumMetaSimulation", "MultiprocessingRepeatedSimulation"]


class _MetaSurvey:
    """The survey of a meta-simulation: only the data counts (``BaseSurvey`` with ``_vnD``)."""

    def __init__(self, vnD):
        self._vnD = [int(n) for n in vnD]

    @property
    def vnD(self):
        return np.asarray(self._vnD)

    @property
    def nD(self):
        return int(sum(self._vnD))


def _in_len(mapping):
    shape = getattr(mapping, "shape", ("*", "*"))
    return shape[1]


def _out_len(mapping):
    shape = getattr(mapping, "shape", ("*", "*"))
    return shape[0]


class MetaSimulation:
    """Several simulations as one: data concatenated, one model through per-child mappings.

    Parameters
    ----------
    simulations : list of simulations (distinct objects)
    mappings : list of maps, one per simulation, all with the same input length
    concurrent : run the children's solves at the same time on their own CUDA
        streams (default: when there is more than one child)
    """

    _repeat_sim = False

    def __init__(self, simulations, mappings, concurrent=None):
        self.simulations = simulations
        self.mappings = mappings
        self.concurrent = (len(self._simulations) > 1) if concurrent is None else bool(concurrent)
        self._model = None
        self._jtjdiag = None
        self._streams = None
        self.survey = self._make_survey()
        self._data_offsets = np.cumsum(np.r_[0, self.survey.vnD])

    # ------------------------------------------------------------ properties
    def _make_survey(self):
        return _MetaSurvey([sim.survey.nD for sim in self.simulations])

    @property
    def simulations(self):
        return self._simulations

    @simulations.setter
    def simulations(self, value):
        value = list(value)
        if not value:
            raise ValueError("simulations must be a non-empty list")
        if len({id(s) for s in value}) != len(value):
            raise ValueError("simulations must be unique")
        self._simulations = value

    @property
    def mappings(self):
        return self._mappings

    @mappings.setter
    def mappings(self, value):
        value = list(value)
        if not self._repeat_sim and len(value) != len(self.simulations):
            raise ValueError("Must provide the same number of mappings and simulations.")
        n_in = _in_len(value[0])
        sims = [self.simulation] * len(value) if self._repeat_sim else self.simulations
        for i, (mapping, sim) in enumerate(zip(value, sims)):
            if _in_len(mapping) != n_in:
                raise ValueError("All mappings must have the same input length")
            out = _out_len(mapping)
            sim_map = getattr(sim, "sigmaMap", None) or getattr(sim, "etaMap", None)
            sim_in = _in_len(sim_map) if sim_map is not None else "*"
            if out != "*" and sim_in != "*" and out != sim_in:
                raise ValueError(f"Simulation and mapping at index {i} inconsistent. Simulation mapping shape "
                                 f"{sim_in} incompatible with input mapping shape {out}.")
        self._mappings = value

    @property
    def model(self):
        return self._model

    @model.setter
    def model(self, value):
        if value is None:
            updated = self._model is not None
            self._model = None
        else:
            value = np.asarray(value, dtype=np.float64).ravel()
            n_in = _in_len(self.mappings[0])
            if n_in != "*" and value.size != n_in:
                raise ValueError(f"model must have {n_in} parameters, got {value.size}")
            updated = self._model is None or self._model.shape != value.shape or not np.array_equal(self._model,
                                                                                                    value)
            if updated:
                self._model = value.copy()
        if updated:
            self._jtjdiag = None
            if not self._repeat_sim:
                for mapping, sim in zip(self.mappings, self.simulations):
                    sim.model = None if value is None else mapping * self._model

    # ------------------------------------------------------------ concurrency
    def _each(self, fn):
        """[fn(i, mapping, sim) for every child], concurrently on the children's own streams."""
        items = list(zip(range(len(self.mappings)), self.mappings, self.simulations))
        if not self.concurrent or self._repeat_sim or len(items) < 2:
            return [fn(*it) for it in items]
        import torch

        if self._streams is None:
            # one stream per child, on the child's own device
            self._streams = [torch.cuda.Stream(device=getattr(sim, "device", None)) for _, _, sim in items]
        caller = torch.cuda.current_stream()
        caller.synchronize()  # inputs the caller produced on its stream are ready for every child

        def run(it):
            s = self._streams[it[0]]
            with torch.cuda.device(s.device), torch.cuda.stream(s):
                out = fn(*it)
            s.synchronize()  # the child's results are complete when its thread returns
            return out

        with ThreadPoolExecutor(max_workers=self._max_workers(len(items))) as ex:
            return list(ex.map(run, items))

    def _max_workers(self, n):
        return n

    # ------------------------------------------------------------ simulation API
    def fields(self, m):
        """The fields of every child (a list) (``simulation.py:194-217``)."""
        self.model = m

        def one(i, mapping, sim):
            if self._repeat_sim and self.model is not None:
                sim.model = mapping * self.model
            return sim.fields(sim.model)

        return self._each(one)

    def dpred(self, m=None, f=None):
        if f is None:
            if m is None:
                m = self.model
            f = self.fields(m)
        out = []
        for i, mapping, sim in zip(range(len(f)), self.mappings, self.simulations):
            if self._repeat_sim:
                sim.model = mapping * self.model
            out.append(sim.dpred(m=sim.model, f=f[i]))
        return self._combine(out)

    def _combine(self, parts):
        return np.concatenate(parts)

    def Jvec(self, m, v, f=None):
        self.model = m
        if f is None:
            f = self.fields(m)

        def one(i, mapping, sim):
            if self._repeat_sim:
                sim.model = mapping * self.model
            return sim.Jvec(sim.model, mapping.deriv(self.model) @ v, f=f[i])

        return self._combine(self._each(one))

    def _data_slice(self, v, i):
        return v[self._data_offsets[i]:self._data_offsets[i + 1]]

    def Jtvec(self, m, v, f=None):
        self.model = m
        if f is None:
            f = self.fields(m)

        def one(i, mapping, sim):
            if self._repeat_sim:
                sim.model = mapping * self.model
            return mapping.deriv(self.model).T @ sim.Jtvec(sim.model, self._data_slice(v, i), f=f[i])

        return sum(self._each(one))

    def _child_weights(self, W, i):
        return sp.diags(self._data_slice(W, i))

    def getJtJdiag(self, m, W=None, f=None):
        """Column norms of J through the mappings (``simulation.py:257-325``)."""
        self.model = m
        if self._jtjdiag is None:
            if W is None:
                W = np.ones(self.survey.nD)
            else:
                try:
                    W = W.diagonal()
                except (AttributeError, TypeError, ValueError):
                    pass
            if f is None:
                f = self.fields(m)

            def one(i, mapping, sim):
                if self._repeat_sim:
                    sim.model = mapping * self.model
                d = sim.getJtJdiag(sim.model, self._child_weights(W, i), f=f[i])
                m_deriv = sp.csr_matrix(mapping.deriv(self.model))
                return np.asarray((sp.diags(np.sqrt(d)) @ m_deriv).power(2).sum(axis=0)).ravel()

            self._jtjdiag = sum(self._each(one))
        return self._jtjdiag


class SumMetaSimulation(MetaSimulation):
    """Data of all children summed (``simulation.py:332-423``): every child has the same
    number of data; ``Jtvec`` passes the whole vector to every child."""

    def _make_survey(self):
        return _MetaSurvey([self.simulations[0].survey.nD])

    @MetaSimulation.simulations.setter
    def simulations(self, value):
        MetaSimulation.simulations.fset(self, value)
        nD = self._simulations[0].survey.nD
        if any(sim.survey.nD != nD for sim in self._simulations):
            raise ValueError("All simulations must have the same number of data.")

    def _combine(self, parts):
        return sum(parts)

    def _data_slice(self, v, i):
        return v

    def _child_weights(self, W, i):
        return sp.diags(W)


class RepeatedSimulation(MetaSimulation):
    """One simulation evaluated under several mappings (``simulation.py:426-520``); the
    evaluations run one after the other (they share the simulation)."""

    _repeat_sim = True

    def __init__(self, simulation, mappings):
        self.simulation = simulation
        super().__init__([simulation], mappings, concurrent=False)

    def _make_survey(self):
        return _MetaSurvey(len(self.mappings) * [self.simulation.survey.nD])

    @property
    def simulations(self):
        return [self.simulation] * len(getattr(self, "_mappings", [None]))

    @simulations.setter
    def simulations(self, value):
        pass

    @property
    def simulation(self):
        return self._simulation

    @simulation.setter
    def simulation(self, value):
        self._simulation = value

    def _each(self, fn):
        return [fn(i, mapping, self.simulation) for i, mapping in enumerate(self.mappings)]


class MultiprocessingMetaSimulation(MetaSimulation):
    """``MetaSimulation`` with at most ``n_processes`` children solving at once
    (``simpeg/meta/multiprocessing.py:31-350``), on CUDA streams of this process."""

    def __init__(self, simulations, mappings, n_processes=None):
        self.n_processes = n_processes
        super().__init__(simulations, mappings, concurrent=True)

    def _max_workers(self, n):
        return n if not self.n_processes else max(1, min(n, int(self.n_processes)))

    def close(self):
        """Nothing to shut down (no worker processes); kept for the reference's API."""


class MultiprocessingSumMetaSimulation(SumMetaSimulation, MultiprocessingMetaSimulation):
    """``SumMetaSimulation`` with at most ``n_processes`` children solving at once."""

    def __init__(self, simulations, mappings, n_processes=None):
        MultiprocessingMetaSimulation.__init__(self, simulations, mappings, n_processes=n_processes)


class MultiprocessingRepeatedSimulation(RepeatedSimulation):
    """``RepeatedSimulation`` under the reference's multiprocessing name (the
    evaluations share one simulation and run one after the other)."""

    def __init__(self, simulation, mappings, n_processes=None):
        self.n_processes = n_processes
        super().__init__(simulation, mappings)

    def close(self):
        """Nothing to shut down (no worker processes); kept for the reference's API."""
