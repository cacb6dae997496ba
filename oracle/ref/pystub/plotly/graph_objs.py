"""plotly.graph_objs stand-in: any trace or layout name is an inert class."""


class _Inert:
    def __init__(self, *args, **kwargs):
        self.args, self.kwargs = args, kwargs


def __getattr__(name):
    return type(name, (_Inert,), {})
