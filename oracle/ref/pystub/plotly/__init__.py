"""Stand-in for the `plotly` Python package, which the reference's NS_kim_
step imports through lib/io/plotly.h (it builds plot objects on its first
step and never draws them) and which is not installed here. Test
infrastructure for the reference harness only: every object it hands out
accepts any arguments and does nothing."""
__version__ = "0-stub"
