"""galax interop: the plum plug-in that lets galax call this library
(``galax_plugin``, loaded by galax through its ``galax.potential.interop`` and
``galax.dynamics.interop`` entry points), and the conversion of galax
potentials into this library's component tables (``convert``)."""
