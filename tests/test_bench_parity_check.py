"""bench.py names every parity object of its JSON line whose agreement count falls short of its checked
count (a mismatch must not pass unnoticed in a long line): agree/checked pairs, the RRTConnect
alone-versus-mix comparison and the PRM edge-list digest."""
import bench


def test_full_agreement_is_clean():
    line = {"parity": {"edges_checked": 20000, "edges_agree": 20000, "knn_checked": 500, "knn_agree": 500},
            "sampling": {"parity": {"values_checked": 10, "values_agree": 10, "compared": "text"}},
            "workloads": {"prm": {"parity": {"digest_match": True, "edges": 5}},
                          "rrt": {"alone_equals_mix": {"clients_checked": 4, "clients_same": 4}}}}
    assert bench.parity_shortfalls(line) == []


def test_each_shortfall_is_named():
    line = {"parity": {"edges_checked": 20000, "edges_agree": 19999, "knn_checked": 500, "knn_agree": 500},
            "sampling": {"parity": {"values_checked": 10, "values_agree": 0}},
            "workloads": {"prm": {"parity": {"digest_match": False}},
                          "rrt": {"alone_equals_mix": {"clients_checked": 4, "clients_same": 3}},
                          "circles": {"parity": {"states_checked": 3, "states_agree": 3}}}}
    assert sorted(bench.parity_shortfalls(line)) == sorted([
        "/parity/edges_checked",
        "/sampling/parity/values_checked",
        "/workloads/prm/parity/digest_match",
        "/workloads/rrt/alone_equals_mix/clients_checked",
    ])
