"""GB300-native VEGAS Monte Carlo integration with the vegasflow API.

Drop-in names (vegasflow __init__.py:3-8): ``VegasFlow``, ``PlainFlow``,
``VegasFlowPlus``, ``vegas_wrapper``, ``vegas_sampler``, ``plain_wrapper``,
``plain_sampler``, ``vegasflowplus_wrapper``, ``vegasflowplus_sampler``,
``float_me``, ``int_me``, ``run_eager``, ``DTYPE``, ``DTYPEINT``.
"""

from .configflow import DTYPE, DTYPEINT, float_me, int_me, run_eager
from .plain import PlainFlow, plain_sampler, plain_wrapper
from .vflow import VegasFlow, vegas_sampler, vegas_wrapper
from .vflowplus import VegasFlowPlus, vegasflowplus_sampler, vegasflowplus_wrapper
from . import integrands

__version__ = "1.4.0+gb300"
