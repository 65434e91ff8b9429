"""GB300-native 2D subset-DIC hot path (Traditional-DIC drop-in).

The directory name contains a hyphen, so the package is registered under the import name
``traditional_dic_gb300`` by ``__graft_entry__.load_package()`` (or any equivalent
``importlib`` spec with ``submodule_search_locations`` set to this directory).
"""
__all__ = ["subset", "synthetic", "build"]
