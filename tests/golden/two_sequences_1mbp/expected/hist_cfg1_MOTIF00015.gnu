set output "hist_cfg1_MOTIF00015.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-33.4977:13.0602]
set yrange [0:130576]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00015.dat" using 1:2 title 'MOTIF00015 (cfg1)' with boxes
