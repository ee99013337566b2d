set output "hist_group1_MOTIF00007.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-46.1868:13.0325]
set yrange [0:131193]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00007.dat" using 1:2 title 'MOTIF00007 (group1)' with boxes
