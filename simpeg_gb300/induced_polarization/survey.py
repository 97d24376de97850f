"""IP survey helpers (``simpeg/electromagnetics/static/induced_polarization/survey.py``)."""

from ..resistivity.survey import Survey

__all__ = ["Survey", "from_dc_to_ip_survey"]


def from_dc_to_ip_survey(dc_survey, dim="2.5D"):
    """IP survey with the DC survey's sources and receivers (``survey.py:5-24``).

    As in the reference, the source list is shared, not copied, and ``dim`` is
    accepted for signature compatibility only."""
    return Survey(dc_survey.source_list)
